"""Malformed-file driver for the Exodus reader, run in a child process by
tests/test_io.py so that a crash fails the test instead of ending pytest.

argv: path of a valid CDF-2 Exodus file, seed.  Every mutated copy must be
either read into a mesh or refused with an fvh_status; the process prints the
counts and exits 0.
"""
import os
import sys
import tempfile

import numpy as np

import flecsale_gb300.hydro as H


def main(path: str, seed: int) -> int:
    data = open(path, "rb").read()
    rng = np.random.default_rng(seed)
    ok = refused = 0
    cases = [data[:n] for n in (0, 3, 4, 8, 12, 40, len(data) // 2, len(data) - 1)]
    header = min(len(data), 600)  # dimensions, attributes and the variable list
    for _ in range(400):
        b = bytearray(data)
        for _ in range(int(rng.integers(1, 5))):
            pos = int(rng.integers(4, header))
            b[pos] = int(rng.integers(0, 256))
        cases.append(bytes(b))
    for _ in range(100):  # whole 32-bit words of the header set to extreme values
        b = bytearray(data)
        pos = int(rng.integers(1, header // 4)) * 4
        b[pos:pos + 4] = int(rng.choice([0, 1, 0x7FFFFFFF, 0xFFFFFFFF, 0x80000000])).to_bytes(4, "big")
        cases.append(bytes(b))
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "m.g")
        for case in cases:
            with open(p, "wb") as f:
                f.write(case)
            try:
                m = H.read_exodus(p)
                assert m.num_cells > 0 and m.dim in (2, 3)
                ok += 1
            except H.FvhError:
                refused += 1
    print(f"read {ok} refused {refused}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1], int(sys.argv[2])))
