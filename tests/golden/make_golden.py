"""Generate the golden fixtures in this directory from the reference tree.

Run once, where the reference checkout is available:
    python tests/golden/make_golden.py /path/to/flecsale
The fixtures are committed; tests never read the reference tree itself.

Outputs
  shock_box_2d_32x32.npz  from apps/hydro/2d/shock_box_2d-solution_rank000000.txt.1procs.std
      vertex_coord (1089,2), cell_centroid (1024,2), cells (1024,5) = density,
      internal_energy, pressure, velocity(0), velocity(1) after 20 steps,
      soln_time, iterations.  The mesh file (data/meshes/square_32x32.g) is
      netCDF-4/HDF5 and unreadable here, so the tests rebuild the mesh from the
      vertex coordinates and centroids listed in the dump.
  ref_physics_vectors.npz  outputs of the reference's own euler_eqns.h /
      flux.h / ideal_gas.h (compiled by oracle/ref_build.py) on seeded random
      states: wall, HLLE and Rusanov fluxes and the per-cell update.
  shock_box_2d_32x32_2procs.npz  from apps/hydro/2d/shock_box_2d-solution_rank00000{0,1}.txt.2procs.std
      (the same problem run on two ranks): per rank the 544 listed cells
      (owned and ghost) as rank{r}_centroid (544,2), rank{r}_cells (544,5)
      in the column order above, rank{r}_global_id; soln_time, iterations.
  shock_box_3d_20x20x20.npz  from apps/hydro/3d/shock_box_3d-solution_rank000000.txt.1procs.std
      and data/meshes/sedov_20x20x20.g (CDF-2, HEX8): exodus_coord (9261,3),
      exodus_connect (8000,8) zero-based, std_cell_centroid (8000,3),
      the uniform final state (density, internal_energy, pressure), the
      largest |velocity| in the dump, soln_time, iterations.
"""
from __future__ import annotations

import os
import sys

import numpy as np


def read_dump(path: str):
    """Parse the reference dump format (apps/hydro/tasks.h:771-849)."""
    cells, verts, header = [], [], {}
    section = None
    with open(path) as fh:
        for line in fh:
            if line.startswith("# Solution time:"):
                header["soln_time"] = float(line.split(":")[1])
            elif line.startswith("# Number iterations:"):
                header["iterations"] = int(line.split(":")[1])
            elif line.startswith("# BEGIN CELLS"):
                section = cells
            elif line.startswith("# BEGIN VERTICES"):
                section = verts
            elif line.startswith("# END"):
                section = None
            elif line.startswith("#") or not line.strip():
                continue
            elif section is not None:
                section.append([float(x) for x in line.split()])
    return header, np.array(cells), np.array(verts)


def main(ref: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    h2, c2, v2 = read_dump(os.path.join(
        ref, "apps/hydro/2d/shock_box_2d-solution_rank000000.txt.1procs.std"))
    assert np.array_equal(c2[:, 0], np.arange(len(c2))) and np.array_equal(v2[:, 0], np.arange(len(v2)))
    np.savez_compressed(
        os.path.join(here, "shock_box_2d_32x32.npz"),
        vertex_coord=v2[:, 2:4], cell_centroid=c2[:, 2:4], cells=c2[:, 4:9],
        soln_time=h2["soln_time"], iterations=h2["iterations"])

    two = {}
    for r in (0, 1):
        hr, cr, _ = read_dump(os.path.join(
            ref, f"apps/hydro/2d/shock_box_2d-solution_rank00000{r}.txt.2procs.std"))
        assert hr["iterations"] == h2["iterations"] and hr["soln_time"] == h2["soln_time"]
        two[f"rank{r}_centroid"] = cr[:, 2:4]
        two[f"rank{r}_cells"] = cr[:, 4:9]
        two[f"rank{r}_global_id"] = cr[:, 1].astype(np.int32)
    np.savez_compressed(os.path.join(here, "shock_box_2d_32x32_2procs.npz"),
                        soln_time=h2["soln_time"], iterations=h2["iterations"], **two)

    h3, c3, v3 = read_dump(os.path.join(
        ref, "apps/hydro/3d/shock_box_3d-solution_rank000000.txt.1procs.std"))
    from scipy.io import netcdf_file
    f = netcdf_file(os.path.join(ref, "data/meshes/sedov_20x20x20.g"), "r", mmap=False)
    coord = np.stack([f.variables[k].data for k in ("coordx", "coordy", "coordz")], 1)
    connect = f.variables["connect1"].data.astype(np.int32) - 1
    f.close()
    for k in (5, 6, 7):
        assert len(np.unique(c3[:, k])) == 1
    np.savez_compressed(
        os.path.join(here, "shock_box_3d_20x20x20.npz"),
        exodus_coord=coord, exodus_connect=connect, std_cell_centroid=c3[:, 2:5],
        density=c3[0, 5], internal_energy=c3[0, 6], pressure=c3[0, 7],
        max_abs_velocity=np.abs(c3[:, 8:11]).max(),
        soln_time=h3["soln_time"], iterations=h3["iterations"])


def physics_cases(dim: int, n: int, seed: int):
    """Random primitive states w = (d, v[dim], p, e, T, a) and unit normals."""
    rng = np.random.default_rng(seed)
    def states():
        w = np.empty((n, dim + 5))
        w[:, 0] = rng.uniform(0.1, 2.0, n)
        w[:, 1:1 + dim] = rng.uniform(-2.0, 2.0, (n, dim))
        w[:, 1 + dim] = rng.uniform(0.05, 3.0, n)
        w[:, 2 + dim] = rng.uniform(0.1, 3.0, n)
        w[:, 3 + dim] = rng.uniform(0.1, 3.0, n)
        w[:, 4 + dim] = rng.uniform(0.3, 2.0, n)
        return w
    wl, wr = states(), states()
    nrm = rng.normal(size=(n, dim))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    du = rng.uniform(-0.01, 0.01, (n, dim + 2))
    return wl, wr, nrm, du


def make_physics_vectors(here: str) -> None:
    """Outputs of the reference's own physics code (oracle/_ref) on seeded
    random inputs: wall/HLLE/Rusanov fluxes and the per-cell update."""
    import ctypes as C
    sys.path.insert(0, os.path.dirname(os.path.dirname(here)))
    from oracle import ref_build
    R = C.CDLL(ref_build.build())
    dp = C.POINTER(C.c_double)
    out = {}
    for dim in (2, 3):
        wl, wr, nrm, du = physics_cases(dim, 64, 100 + dim)
        for kind in (-1, 0, 1):
            f = np.zeros((len(wl), dim + 2))
            for i in range(len(wl)):
                R.ref_face_flux(dim, kind, *(np.ascontiguousarray(x).ctypes.data_as(dp)
                                             for x in (wl[i], wr[i], nrm[i], f[i])))
            out[f"flux_{dim}d_{kind}"] = f
        w = wl.copy()
        for i in range(len(w)):
            row = np.ascontiguousarray(w[i])
            R.ref_update_cell(dim, C.c_double(1.4), C.c_double(1.0), row.ctypes.data_as(dp),
                              np.ascontiguousarray(du[i]).ctypes.data_as(dp))
            w[i] = row
        out[f"update_{dim}d"] = w
    np.savez_compressed(os.path.join(here, "ref_physics_vectors.npz"), **out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FLECSALE_REFERENCE", "")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set FLECSALE_REFERENCE)")
    os.environ["FLECSALE_REFERENCE"] = ref
    main(ref)
    make_physics_vectors(os.path.dirname(os.path.abspath(__file__)))
