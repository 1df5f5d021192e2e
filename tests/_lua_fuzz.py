"""Mutated input files for the Lua-subset interpreter, run in a child process
by tests/test_input.py so that a crash fails the test instead of ending
pytest.  argv: seed, count.  Each mutant of the shipped input files (bytes
replaced, inserted or deleted, or the file cut short) must load, or be
refused with an fvh_status; the process prints the counts and exits 0."""
import os
import sys

import numpy as np

import flecsale_gb300.hydro as H

HERE = os.path.dirname(os.path.abspath(__file__))
ALPHABET = list(b"()[]{}=.,;:+-*/%^#<>~\"'\\\n 0123456789aefxnilortudhws_") + [0, 128, 255]


def main(seed: int, count: int) -> int:
    srcs = [open(os.path.join(HERE, "golden", "inputs", f), "rb").read()
            for f in ("shock_box_2d.lua", "shock_box_3d_box.lua")]
    rng = np.random.default_rng(seed)
    mesh = H.HostMesh.box(2, (4, 3), [0, 0], [1, 1])
    loaded = refused = 0
    for it in range(count):
        b = bytearray(srcs[it % 2])
        for _ in range(int(rng.integers(1, 6))):
            if not b:
                break
            op, pos = int(rng.integers(0, 4)), int(rng.integers(0, len(b)))
            if op == 0:
                b[pos] = int(rng.choice(ALPHABET))
            elif op == 1:
                b.insert(pos, int(rng.choice(ALPHABET)))
            elif op == 2:
                del b[pos]
            else:
                del b[pos:]
        try:
            inp = H.Input(text=bytes(b).decode("latin-1"))
        except H.FvhError:
            refused += 1
            continue
        loaded += 1
        for call in (lambda: inp.initial_state(mesh, inp.params(2)[0]), inp.mesh):
            try:
                call()
            except H.FvhError:
                pass
    print(f"loaded {loaded} refused {refused}")
    return 0


if __name__ == "__main__":
    sys.exit(main(int(sys.argv[1]), int(sys.argv[2])))
