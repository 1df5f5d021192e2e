"""The oracle's own box-mesh builder (oracle/box_mesh.cpp) against the
product's general mesh builder: identical arrays, bit for bit.

The benchmark's CPU baseline builds its workload with the oracle's builder so
that it never loads the product library; this test is what makes the two
workloads the same.  The four-quadrant initial state built on the oracle side
is checked against the product's initial-condition routine the same way.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
import oracle


@pytest.mark.parametrize("n,jitter,seed,lo,hi", [
    ((1, 1), 0.0, 0, (0, 0), (1, 1)),
    ((1, 7), 0.2, 3, (0, 0), (1, 1)),
    ((9, 1), 0.2, 3, (0, 0), (1, 1)),
    ((24, 17), 0.2, 7, (0, 0), (1, 1)),
    ((100, 10), 0.0, 0, (0, 0), (1, 0.1)),
    ((64, 48), 0.3, 11, (-1, 2), (3, 2.5)),
])
def test_box_mesh_equals_product_builder(n, jitter, seed, lo, hi):
    mine = oracle.BoxMesh2D(n[0], n[1], lo, hi, jitter, seed)
    prod = H.HostMesh.box(2, n, list(lo), list(hi), jitter, seed)
    assert (mine.num_cells, mine.num_faces, mine.num_vertices) == \
        (prod.num_cells, prod.num_faces, prod.num_vertices)
    a, b = mine.arrays(), prod.arrays()
    assert set(a) == set(b)
    for k in a:
        assert np.array_equal(a[k], np.asarray(b[k]).reshape(a[k].shape)), k


def test_box_mesh_full_size_equals_product_builder():
    """The benchmark's own mesh: 1024x1024, jitter 0.2h, seed 1."""
    mine = oracle.BoxMesh2D(1024, 1024, (0, 0), (1, 1), 0.2, 1)
    prod = H.HostMesh.box(2, (1024, 1024), [0, 0], [1, 1], 0.2, 1)
    a, b = mine.arrays(), prod.arrays()
    for k in a:
        assert np.array_equal(a[k], np.asarray(b[k]).reshape(a[k].shape)), k


def test_four_quadrant_state_equals_product_initial_state():
    mine = oracle.BoxMesh2D(48, 40, (0, 0), (1, 1), 0.2, 1)
    prod = H.HostMesh.box(2, (48, 40), [0, 0], [1, 1], 0.2, 1)
    p = H.make_params(2, flux="hllc", cfl=0.4, boundary="outflow")
    assert np.array_equal(oracle.four_quadrant_state(mine), H.initial_state("four_quadrant", prod, p))


def test_oracle_runs_on_its_own_mesh_like_on_the_product_mesh():
    """The same steps on the oracle-built mesh and the product-built mesh give
    the same bits (the oracle's entry points take either structure)."""
    mine = oracle.BoxMesh2D(40, 30, (0, 0), (1, 1), 0.2, 1)
    prod = H.HostMesh.box(2, (40, 30), [0, 0], [1, 1], 0.2, 1)
    po = oracle.params(2, flux="hllc", cfl=0.4, boundary="outflow", final_time=1e9)
    s1 = oracle.four_quadrant_state(mine)
    s2 = s1.copy()
    assert oracle.run(mine, s1, po, 5)[0] == 0
    assert oracle.run(prod, s2, po, 5)[0] == 0
    assert np.array_equal(s1, s2)
