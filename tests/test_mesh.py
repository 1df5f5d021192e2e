"""Topology and geometry of the host mesh builder (the burton queries the hydro
tasks use: cells(f), faces(c), cell_vertex_neighbors(c), vertices(c), centroids,
volumes, face normals and areas)."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H


def _closure(m):
    """Sum over faces(c) of +-A_f n_f must vanish for a closed cell."""
    a = m.arrays()
    off, cf = a["cell_face_offsets"], a["cell_faces"]
    s = np.zeros((m.dim, m.num_cells))
    for c in range(m.num_cells):
        for q in range(off[c], off[c + 1]):
            f = cf[q]
            sign = 1.0 if f >= 0 else -1.0
            f = f if f >= 0 else ~f
            s[:, c] += sign * a["face_area"][f] * a["face_normal"][:, f]
    return s


@pytest.mark.parametrize("dim,n,jit", [(2, (9, 7), 0.0), (2, (9, 7), 0.2), (3, (5, 4, 3), 0.0), (3, (5, 4, 3), 0.15)])
def test_box_mesh_invariants(fvh, dim, n, jit):
    m = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, jit, 4)
    a = m.arrays()
    nc = int(np.prod(n))
    assert m.num_cells == nc
    assert m.num_vertices == int(np.prod([k + 1 for k in n]))
    if dim == 2:
        nfaces = (n[0] + 1) * n[1] + n[0] * (n[1] + 1)
    else:
        nfaces = ((n[0] + 1) * n[1] * n[2] + n[0] * (n[1] + 1) * n[2] + n[0] * n[1] * (n[2] + 1))
    assert m.num_faces == nfaces
    np.testing.assert_allclose(a["cell_volume"].sum(), 1.0, rtol=1e-12)
    assert np.all(a["cell_volume"] > 0)
    np.testing.assert_allclose(np.linalg.norm(a["face_normal"], axis=0), 1.0, rtol=1e-14)
    assert np.abs(_closure(m)).max() < 1e-14
    fc = a["face_cells"]
    assert np.all(fc[:, 0] >= 0) and np.all((fc[:, 1] == -1) | (fc[:, 1] > fc[:, 0]))
    # normals point out of cells(f)[0]
    d = a["face_centroid"] - a["cell_centroid"][:, fc[:, 0]]
    assert np.all(np.sum(d * a["face_normal"], axis=0) > 0)
    # faces get ids in order of first encounter (cell order, then local order)
    first = []
    seen = set()
    for c in range(nc):
        for q in range(a["cell_face_offsets"][c], a["cell_face_offsets"][c + 1]):
            f = a["cell_faces"][q]
            f = f if f >= 0 else ~f
            if f not in seen:
                seen.add(f)
                first.append(f)
    assert first == list(range(m.num_faces))
    # vertex neighbours: all cells sharing a vertex, ascending, no self
    cv = [set(a["cell_vertices"][a["cell_vertex_offsets"][c]:a["cell_vertex_offsets"][c + 1]]) for c in range(nc)]
    for c in range(0, nc, max(1, nc // 13)):
        got = list(a["cell_nbrs"][a["cell_nbr_offsets"][c]:a["cell_nbr_offsets"][c + 1]])
        exp = sorted(k for k in range(nc) if k != c and cv[k] & cv[c])
        assert got == exp
    # boundary vertices stay on the boundary
    vc = a["vertex_coord"]
    assert vc.min() == 0.0 and vc.max() == 1.0


def test_jitter_is_seeded_and_bounded(fvh):
    a = H.HostMesh.box(2, (20, 20), [0, 0], [1, 1], 0.2, 1).arrays()["vertex_coord"]
    b = H.HostMesh.box(2, (20, 20), [0, 0], [1, 1], 0.2, 1).arrays()["vertex_coord"]
    c = H.HostMesh.box(2, (20, 20), [0, 0], [1, 1], 0.2, 2).arrays()["vertex_coord"]
    u = H.HostMesh.box(2, (20, 20), [0, 0], [1, 1], 0.0, 1).arrays()["vertex_coord"]
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.abs(a - u).max() <= 0.2 / 20 + 1e-15 and np.abs(a - u).max() > 0.15 / 20


def test_affine_centroids(fvh):
    """Polygon/hex centroid and volume are exact for affine cells."""
    m = H.HostMesh.box(2, (3, 2), [0, 0], [3, 1], 0.0, 0)
    np.testing.assert_allclose(m.arrays()["cell_centroid"][:, 0], [0.5, 0.25], atol=1e-15)
    m = H.HostMesh.box(3, (2, 2, 2), [0, 0, 0], [2, 4, 6], 0.0, 0)
    a = m.arrays()
    np.testing.assert_allclose(a["cell_volume"], 6.0, rtol=1e-14)
    np.testing.assert_allclose(a["cell_centroid"][:, 0], [0.5, 1.0, 1.5], rtol=1e-14)


def test_tet_mesh(fvh):
    """Two tetrahedra sharing a face (Exodus TETRA4 order)."""
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], float)
    cells = np.array([0, 1, 2, 3, 1, 2, 3, 4][:4] + [1, 4, 2, 3], np.int32)
    m = H.HostMesh.from_cells(3, x, np.array([0, 4, 8], np.int32), cells)
    a = m.arrays()
    assert m.num_faces == 7
    assert np.sum(a["face_cells"][:, 1] >= 0) == 1
    np.testing.assert_allclose(a["cell_volume"][0], 1 / 6, rtol=1e-14)


def test_box_beyond_int32_connectivity_is_refused(fvh):
    """Meshes whose int32 CSR would overflow are refused before any
    allocation: 2D 23171^2 cells need 4 * 5.4e8 > 2^31 cell-vertex entries;
    3D 820^3 cells need 8 * 5.5e8."""
    for dim, n in ((2, (23171, 23171)), (3, (820, 820, 820))):
        with pytest.raises(H.FvhError) as e:
            H.HostMesh.box(dim, n, [0] * dim, [1] * dim)
        assert e.value.code == H.ERR_CAPACITY


def test_box_rejects_empty_and_inverted_extents(fvh):
    for n, lo, hi in (((0, 4), [0, 0], [1, 1]), ((4, 4), [0, 0], [1, 0]),
                      ((4, -1), [0, 0], [1, 1])):
        with pytest.raises(H.FvhError) as e:
            H.HostMesh.box(2, n, lo, hi)
        assert e.value.code == H.ERR_INVALID_ARGUMENT


_OOM_CHILD = r'''
import ctypes as C
import resource
import numpy as np
import flecsale_gb300.hydro as H

L = H.lib()
resource.setrlimit(resource.RLIMIT_AS, (3 << 30, 3 << 30))
h = C.c_void_p()
lo, hi = np.zeros(3), np.ones(3)
# 20000^2 quads: ~6.4 GB of vertex coordinates alone, far beyond the 3 GB limit
rc_box = L.fvh_host_mesh_box(2, np.array([20000, 20000, 1], np.int32).ctypes.data_as(H._ip),
                             H._dptr(lo), H._dptr(hi), 0.0, C.c_uint64(0), C.byref(h))
print("box", rc_box, flush=True)
# the library still works after the failures
m = H.HostMesh.box(2, (8, 8), [0, 0], [1, 1])
print("after", m.num_cells, flush=True)
'''


def test_host_allocation_failure_is_a_status_not_an_abort():
    """A host allocation that fails inside a C entry point returns
    FVH_ERR_OUT_OF_MEMORY instead of letting std::bad_alloc cross the C ABI
    (which would terminate the caller); checked in a child process whose
    address space is capped."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _OOM_CHILD], capture_output=True, text=True,
                       timeout=300, cwd=root, env=dict(os.environ, PYTHONPATH=root,
                                                       OMP_NUM_THREADS="2"))
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    lines = dict(l.split(" ", 1) for l in r.stdout.splitlines())
    assert int(lines["box"]) == H.ERR_OUT_OF_MEMORY
    assert int(lines["after"]) == 64


def _polys(coords, cells):
    off = np.cumsum([0] + [len(c) for c in cells]).astype(np.int32)
    return H.HostMesh.from_cells(2, np.asarray(coords, float), off,
                                 np.concatenate(cells).astype(np.int32))


def test_invalid_polygon_meshes_are_refused(fvh):
    """Meshes whose faces would not close a cell are refused instead of
    giving a non-conservative update: a vertex listed twice in a cell, two
    cells sharing two edges, a cell edge lying across another cell (either
    cell order) and an edge of zero length."""
    sq = [[0, 0], [1, 0], [1, 1], [0, 1]]
    ok = _polys(sq + [[2, 0]], [[0, 1, 2, 3], [1, 4, 2]])
    assert ok.num_cells == 2 and ok.num_faces == 6
    cases = {
        "repeated_vertex": (sq + [[2, 0]], [[0, 1, 2, 3], [1, 4, 2, 2]]),
        "two_shared_edges": ([[0, 0], [2, 0], [1, 1], [2, 2], [0, 2]], [[0, 1, 2, 3, 4], [1, 3, 2]]),
        "edge_across_a_cell": (sq + [[0, 2]], [[0, 1, 2, 3], [0, 2, 4]]),
        "edge_across_a_cell_first": (sq + [[0, 2]], [[0, 2, 4], [0, 1, 2, 3]]),
        "zero_length_edge": (sq + [[1, 0]], [[0, 4, 1, 2, 3]]),
    }
    for name, (coords, cells) in cases.items():
        with pytest.raises(H.FvhError) as e:
            _polys(coords, cells)
        assert e.value.code in (H.ERR_INVALID_ARGUMENT, H.ERR_UNSUPPORTED), name
