#!/usr/bin/env python
"""Benchmark: zone-updates/s of the Eulerian MUSCL hydro step on GB300.

Workload (one bench step = one full time step: CFL dt reduction + predictor +
corrector, apps/hydro/driver.h:325-375): 2D four-quadrant Riemann problem on a
1024x1024 quad mesh over [0,1]^2, interior nodes jittered by a seeded uniform
+-0.2h (seed 1), stored unstructured; ideal gas gamma 1.4; second-order MUSCL
with least-squares vertex-neighbour gradients and the reference's
Barth-Jespersen vertex limiter; HLLC fluxes; transmissive boundaries (with the
reference's reflecting walls the receding SW quadrant empties the corner and
the state goes negative within ~10-80 steps); CFL 0.4.  Synthetic data.

The headline value is the plain FP64 path, whose arithmetic is bitwise the
reference's (the same precision as the reference CPU solver it is compared
with).  Beside it: the mixed-precision form (FP32 reconstruction + flux, FP64
state/update/dt) with its L1/Linf density and energy errors against FP64 after
the same steps; the 512-problem batch; the served request stream (60 s of
Poisson arrivals); the 192^3 3D shock box in both forms; and the CPU baseline.
Every form is also timed end to end through the C ABI from host memory.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (torchrun) runs one independent replica per GPU (the single-mesh step is
not sharded): value = all ranks' zone-updates / max-over-ranks time.
--impl reference times the CPU restatement of the reference solver (the
reference itself cannot be built) with all host threads, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "zone-updates/s on 1 GB300: FP64 plain vs mixed/batched at ≤1e-4 L1; p50/p99"
UNIT = "zone-updates/s"
N_SIDE = 1024
JITTER, SEED = 0.2, 1
WORKLOAD = ("2D four-quadrant Riemann problem, 1024x1024 quads on [0,1]^2 jittered "
            "+-0.2h (seed 1), gamma 1.4, MUSCL LSQ + Barth-Jespersen vertex limiter, "
            "HLLC, transmissive boundaries, CFL 0.4, one step = dt + predictor + corrector")


# the workload's solver settings (the oracle takes the same keywords)
ORACLE_KW = dict(flux="hllc", limiter="barth_jespersen", order=2, swap=True, cfl=0.4,
                 final_time=1.0e9, boundary="outflow")


def build_problem(n_side: int = N_SIDE):
    import flecsale_gb300.hydro as H
    mesh = H.HostMesh.box(2, (n_side, n_side), [0, 0], [1, 1], JITTER, SEED)
    p64 = H.make_params(2, precision="fp64", **ORACLE_KW)
    p32 = H.make_params(2, precision="mixed", **ORACLE_KW)
    state0 = H.initial_state("four_quadrant", mesh, p64)
    return H, mesh, p64, p32, state0


def workload_config(mesh) -> dict:
    """The bench line's config: the same dict for this repository's arm and
    the reference arm (the per-step working set, FP64 state + gradients +
    fluxes + mesh, is far above the 129 MB L2, so no flush is needed)."""
    ws_mb = 1572 * mesh.num_cells / 2 / 1e6
    return {"workload": WORKLOAD, "cells": mesh.num_cells, "faces": mesh.num_faces,
            "form": "plain FP64",
            "l2": (f"no flush: per-stage working set ~{ws_mb:.0f} MB > 129 MB L2" if ws_mb > 129
                   else f"small test size: per-stage working set ~{ws_mb:.0f} MB fits in L2")}


def conservation_totals(mesh, state) -> dict:
    """Mass, momentum and total energy of a state: FP64 sums over cells of the
    conserved variables (rho, rho v, rho (e + |v|^2 / 2)) times the cell
    volumes."""
    D = mesh.dim
    vol = mesh.arrays()["cell_volume"]
    d, v, e = state[0], state[1:1 + D], state[1 + D]
    return {"mass": float(np.dot(d, vol)),
            "momentum": [float(np.dot(d * v[k], vol)) for k in range(D)],
            "energy": float(np.dot(d * (e + 0.5 * (v * v).sum(axis=0)), vol))}


# ---------------------------------------------------------------------------
# algorithmic bytes per launch (each array a kernel must touch, moved once)
# ---------------------------------------------------------------------------
def algorithmic_bytes(mesh, precision: str) -> dict:
    D = mesh.dim
    nc, nf, nv = mesh.num_cells, mesh.num_faces, mesh.num_vertices
    ncf, nnb, ncv = mesh.nnz_faces, mesh.nnz_nbrs, mesh.nnz_vertices
    csr_cf = 4 * (nc + 1) + 4 * ncf
    csr_nb = 4 * (nc + 1) + 4 * nnb
    csr_cv = 4 * (nc + 1) + 4 * ncv
    if precision == "fp64":
        return {
            "dt": nc * (8 * (1 + D) + 8) + csr_cf + nf * (8 * D + 8),
            "gradients": 8 * (D + 4) * nc + 8 * D * nc + 8 * D * nv + csr_nb + csr_cv
                         + 8 * D * (D + 4) * nc,
            "fluxes": 8 * nf + 8 * D * nf * 2 + 8 * nf + 8 * (D + 2) * nf
                      + 8 * (D + 4) * nc + 8 * D * (D + 4) * nc + 8 * D * nc,
            "update": csr_cf + 8 * (D + 2) * nf + 8 * nc + 8 * (D + 2) * nc + 8 * (D + 5) * nc,
        }
    cen4 = 1 if D == 2 else 2
    grad4 = 3 if D == 2 else 6
    fdx4 = 1 if D == 2 else 2      # face offsets; also the face-flux record size
    del4 = 2 if D == 2 else 3      # predictor increments (double-float)
    state_in = 8 * (D + 2) * nc    # FP64 d, v, e read by an update
    face_geo = 8 * nf + 16 * nf + 16 * fdx4 * nf  # face cells, normal+area, offsets
    recon_in = 32 * nc + 16 * grad4 * nc           # FP32 pack + gradients
    pred_out = 16 * del4 * nc + 32 * nc            # increments + next pack
    corr_io = 16 * del4 * nc + 8 * (D + 5) * nc    # increments in, FP64 state out
    b = {
        # FP64 state in (d, v, e, p, a), FP32 pack out, inv_vol32, faces, face geometry
        "pack_dt": 8 * (D + 4) * nc + 32 * nc + 4 * nc + csr_cf + 16 * nf,
        # pack + centroid per cell, neighbour CSR, cell-vertex CSR + vertex
        # coordinates (hi/lo) for the limiter, gradients out
        "gradients": 32 * nc + 16 * cen4 * nc + csr_nb + csr_cv + 16 * cen4 * nv
                     + 16 * grad4 * nc,
        # schedule 0: fluxes evaluated by each cell, then the update
        "flux_update_predictor": recon_in + csr_cf + face_geo + 8 * nc + state_in + pred_out,
        "flux_update_corrector": recon_in + csr_cf + face_geo + 8 * nc + state_in + corr_io,
        # schedule 1: face-flux array, then the cell gather + update
        "face_flux": recon_in + face_geo + 16 * fdx4 * nf,
        "gather_update_predictor": csr_cf + 16 * fdx4 * nf + 8 * nc + state_in + pred_out,
        "gather_update_corrector": csr_cf + 16 * fdx4 * nf + 8 * nc + state_in + corr_io,
    }
    # inside a run the corrector also writes the next step's pack and finds
    # its CFL maximum (1/V in FP32; the face geometry, already read by a
    # schedule-0 corrector), so later steps have no pack_dt
    b["flux_update_corrector_next"] = b["flux_update_corrector"] + 32 * nc + 4 * nc
    b["gather_update_corrector_next"] = b["gather_update_corrector"] + 32 * nc + 4 * nc + 16 * nf
    # schedule 2 (face colouring): all colours of a stage together (the face
    # kernel's reads plus a read-modify-write of each side's sums, 2(D+2)
    # floats), and the update from the sums
    acc = 4 * 2 * (D + 2)
    b["face_colour_stage"] = recon_in + face_geo + 2 * 2 * acc * nf
    b["colour_update"] = (8 * nc + state_in + pred_out + 2 * acc * nc
                          + 8 * nc + state_in + corr_io + 2 * acc * nc + 32 * nc + 4 * nc
                          + 16 * nf) / 2
    # the profile reports one mean per kernel name over both stages of a run
    b["flux_update"] = (b["flux_update_predictor"] + b["flux_update_corrector_next"]) / 2
    b["gather_update"] = (b["gather_update_predictor"] + b["gather_update_corrector_next"]) / 2
    return b


def per_zone_update_bytes(mesh, precision: str) -> float:
    b = algorithmic_bytes(mesh, precision)
    if precision == "fp64":
        tot = b["dt"] + 2 * (b["gradients"] + b["fluxes"] + b["update"])
    else:
        # a step of a run (schedule 0, no face-flux array): the minimum traffic
        tot = 2 * b["gradients"] + b["flux_update_predictor"] + b["flux_update_corrector_next"]
    return tot / mesh.num_cells


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic() -> dict:
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary: {form:kernel: {"bytes", "commit", ...}}."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
    except Exception:
        return {}
    return {k: (v if isinstance(v, dict) else {"bytes": v}) for k, v in d.items()}


def ncu_pipes() -> dict:
    """Per-kernel pipe utilisation (fractions) from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "pipe_utilization.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.out = gpu, None, None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self) -> dict:
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (C++ restatement of the reference, OpenMP)
# ---------------------------------------------------------------------------
def cpu_baseline(n_side: int, budget_s: float = 12.0, max_steps: int = 400) -> dict:
    """The oracle (the reference's tasks restated in C++/OpenMP) on the host
    cores, on the same workload built by the oracle's own mesh builder: all
    threads (the reported value) and one thread."""
    import oracle
    O = oracle.load()
    mesh = oracle.BoxMesh2D(n_side, n_side, (0.0, 0.0), (1.0, 1.0), JITTER, SEED)
    p64 = oracle.params(2, **ORACLE_KW)
    state0 = oracle.four_quadrant_state(mesh)

    def sample(budget):
        s = state0.copy()
        oracle.run(mesh, s, p64, 1)  # warm-up step
        n, t0 = 0, time.perf_counter()
        while n < max_steps and (time.perf_counter() - t0) < budget:
            oracle.run(mesh, s, p64, 1)
            n += 1
        return n, time.perf_counter() - t0

    O.oracle_set_threads(0)
    cores = int(O.oracle_max_threads())
    n, dt = sample(budget_s)
    O.oracle_set_threads(1)
    n1, dt1 = sample(budget_s / 3)
    O.oracle_set_threads(0)
    return {"value": mesh.num_cells * n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} full time steps of the {n_side}x{n_side} workload in {dt:.1f} s "
                      f"(FP64, HLLC; oracle/hydro_oracle.cpp, -O2, OpenMP)",
            "one_thread": {"value": mesh.num_cells * n1 / dt1, "cores": 1,
                           "sample": f"{n1} steps in {dt1:.1f} s"}}


# ---------------------------------------------------------------------------
def dist_setup(backend: str):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
        return dist, ws, rank, local
    return None, 1, 0, local


def max_over_ranks(dist, value: float, device: str = "cuda") -> float:
    """Maximum of a per-rank time over all ranks (all-reduce MAX); identity
    without a process group."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """The reference arm: the CPU restatement of the reference solver (the
    reference itself cannot be built) on the same workload, all host threads,
    rank 0 only.  Mesh, initial state and parameters come from the oracle's own
    builders, so this process never loads the product library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    mesh = oracle.BoxMesh2D(args.n, args.n, (0.0, 0.0), (1.0, 1.0), JITTER, SEED)
    p64 = oracle.params(2, **ORACLE_KW)
    s = oracle.four_quadrant_state(mesh)
    O = oracle.load()
    O.oracle_set_threads(0)
    for _ in range(args.warmup):
        oracle.run(mesh, s, p64, 1)
    t0 = time.perf_counter()
    st, _, _ = oracle.run(mesh, s, p64, args.steps)
    dt = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError(f"reference arm: oracle status {st}")
    cores = int(O.oracle_max_threads())
    value = mesh.num_cells * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(mesh),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full time steps of the workload after "
                                   f"{args.warmup} warm-up steps, all host threads "
                                   "(oracle/hydro_oracle.cpp, -O2, OpenMP; mesh from "
                                   "oracle/box_mesh.cpp)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


BATCH_PROBLEMS, BATCH_SEED = 512, 3
BATCH_KINDS = ("kelvin_helmholtz", "four_quadrant", "sod")


def batch_problems(n=BATCH_PROBLEMS, seed=BATCH_SEED):
    """Sizes log-uniform in [32^2, 512^2] cells (side log-uniform in [32, 512]),
    jitter +-0.2h, problem kinds cycling KH shear layer / four-quadrant / Sod."""
    import flecsale_gb300.hydro as H
    rng = np.random.default_rng(seed)
    sides = np.exp(rng.uniform(np.log(32), np.log(512), n)).round().astype(int)
    return [(H.HostMesh.box(2, (int(s), int(s)), [0, 0], [1, 1], JITTER, 1000 + k),
             BATCH_KINDS[k % 3]) for k, s in enumerate(sides)]


def run_batched(torch, stream, steps: int, warmup: int) -> dict:
    """The batched form: all problems advanced by one CUDA-graph launch per
    step, per-problem dt, launch shape picked by the autotuner."""
    import flecsale_gb300.hydro as H
    t0 = time.perf_counter()
    from flecsale_gb300 import serve
    probs = batch_problems()
    p = serve.server_params()
    meshes = [m for m, _ in probs]
    b = H.Batch.for_meshes(p, meshes)
    b.assign(meshes, 0.4, 1.0e9, stream=stream)
    for k, (m, kind) in enumerate(probs):
        b.set_state(k, H.initial_state(kind, m, p, seed=k), 0.0, stream)
    setup_s = time.perf_counter() - t0
    tune = b.autotune(trial_steps=3, use_cache=False, stream=stream)
    for _ in range(warmup):
        b.step(1, stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(steps, stream)  # one graph launch advances every problem `steps` steps
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    _, codes, _ = b.query(stream)
    if np.any(codes != 0):
        raise RuntimeError(f"batched: device status {codes[codes != 0][:4]}")
    nc = b.num_cells
    # accuracy: sampled problems (smallest, median, largest) rerun alone in FP64
    # for the same number of steps
    sizes = [m.num_cells for m in meshes]
    order = np.argsort(sizes)
    acc = []
    p64 = H.make_params(2, flux="hllc", precision="fp64", boundary="outflow", swap=False,
                        cfl=0.4, final_time=1.0e9)
    E = lambda s: s[0] * (s[3] + 0.5 * (s[1] ** 2 + s[2] ** 2))
    for k in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
        m, kind = probs[k]
        dm, ds = H.DeviceMesh(m), H.DeviceState(2, m.num_cells)
        sol = H.Solver(dm, p64)
        ds.upload(H.initial_state(kind, m, p64, seed=k), stream)
        sol.reset(0.0, stream)
        sol.run(ds, warmup + steps, stream=stream)  # the autotuner restores the state
        ref, mix = ds.download(stream), b.get_state(k, stream)
        acc.append({"problem": k, "cells": m.num_cells, "kind": kind,
                    "l1_density": float(np.abs(mix[0] - ref[0]).sum() / np.abs(ref[0]).sum()),
                    "linf_density": float(np.abs(mix[0] - ref[0]).max()),
                    "l1_total_energy": float(np.abs(E(mix) - E(ref)).sum() / np.abs(E(ref)).sum()),
                    "linf_total_energy": float(np.abs(E(mix) - E(ref)).max())})
    return {"value": nc * steps / (ms * 1e-3), "unit": UNIT, "problems": len(meshes),
            "cells": nc, "steps": steps, "ms_per_step": ms / steps,
            "launches": "one CUDA graph launch for all steps",
            "gpu_launches": b.launches_per_step() * steps + 1,  # + the first step's pack
            "autotuned_shape": tune, "host_setup_s": setup_s,
            "tuned_space": "block 128/256 x cells per thread 1/2 x gather schedule 0 (cell-centric "
                           "fluxes) / 1 (face-flux array); the face-colouring schedule is not a "
                           "batch candidate: its per-colour launches scatter over the whole "
                           "concatenated mesh (2.6x slower than gather on one 1024^2 mesh) and "
                           "a batch reassignment would have to recolour it on the host",
            "accuracy_vs_fp64": acc,
            "config": "512 independent 2D problems, cells log-uniform in [32^2, 512^2] (seed 3), "
                      "KH shear layer / four-quadrant / Sod, HLLC, outflow, textbook reconstruction, CFL 0.4, "
                      "mixed precision"}


def run_serving(torch, stream, batched_rate: float, seconds: float, seed: int = 4) -> dict:
    """Poisson arrivals of 2D KH / four-quadrant / Sod requests (sides
    log-uniform 64..2048, end times uniform 0.05..0.3) at a rate that loads the
    device to ~80% of its measured batched throughput; continuous batching."""
    import flecsale_gb300.hydro as H
    from flecsale_gb300 import serve
    # mean work per request ~ 6 * E[side^3] * E[t_end] zone-updates (dt ~ 0.4 h / 2.4)
    lo, hi = 64.0, 2048.0
    e_side3 = (hi ** 3 - lo ** 3) / (3.0 * np.log(hi / lo))
    work = 6.0 * e_side3 * 0.175
    rate = 0.8 * batched_rate / work
    reqs = serve.poisson_requests(rate, seconds, seed)
    p = serve.server_params()
    srv = serve.Server(p, max_cells=48_000_000, max_faces=97_000_000, max_vertices=49_000_000,
                       max_problems=512, steps_per_launch=8, stream=stream)
    rep = srv.run(reqs, time_limit=seconds + 120.0)
    srv.close()
    done = rep.pop("done")
    small = sorted(done, key=lambda r: r.side)[:3]
    l1 = [serve.fp64_rerun_l1(r, p) for r in small]
    rep.update({"arrival_rate_per_s": rate, "arrival_window_s": seconds,
                "l1_density_vs_fp64_rerun": {"requests": [r.side for r in small],
                                             "max": max(l1) if l1 else None},
                "config": "Poisson arrivals at ~80% of the measured batched throughput; sides "
                          "log-uniform 64..2048 (cells 64^2..2048^2), t_end uniform [0.05, 0.3]; "
                          "admission by device capacity (48M cells); 8 steps per graph launch"})
    return rep


def roofline_3d(mesh, form: str, prof: dict, in_run_step_ms: float) -> dict:
    """Dominant kernel of a 3D form against HBM: the reference dataflow's bytes
    of its task (the plain form's per-cell figures, 412 B/cell for the
    gradients in 3D), the duration its profiled share of the in-run step."""
    hbm, peak_kind = peaks()
    ab = algorithmic_bytes(mesh, "fp64")
    task = {"gradients": "gradients", "fluxes": "fluxes", "update": "update", "dt": "dt",
            "face_flux": "fluxes", "gather_update": "update", "pack_dt": "dt"}
    profiled = sum(v[0] * v[1] for v in prof.values())
    scale = in_run_step_ms / profiled
    dom = max(prof, key=lambda k: prof[k][0] * prof[k][1])
    dur = prof[dom][0] * scale
    sb = ab[task[dom]]
    return {"bound": "hbm", "kernel": dom, "duration_ms": dur,
            "algorithmic_bytes_per_launch": sb,
            "bytes_basis": f"reference-dataflow bytes of the {task[dom]} task "
                           f"({sb / mesh.num_cells:.0f} B/cell)",
            "achieved": sb / (dur * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
            "frac": sb / (dur * 1e-3) / 1e9 / hbm, "peak_source": peak_kind,
            "kernels": {k: {"duration_ms": v[0] * scale, "launches_per_step": v[1],
                            "share": v[0] * v[1] / profiled} for k, v in prof.items()}}


def run_3d(torch, stream, n: int = 192, steps: int = 100, shape: str = "") -> dict:
    """192^3 hex shock box (inner cube [0,0.5]^3 at rho=1,p=1, rest 0.125/0.1),
    jitter +-0.15h (seed 2), Rusanov, CFL 0.3, 100 steps: FP64 vs mixed.  The
    mixed form's launch shape is autotuned unless `shape` ("block,cpt,schedule")
    fixes it."""
    import flecsale_gb300.hydro as H
    t0 = time.perf_counter()
    mesh = H.HostMesh.box(3, (n, n, n), [0, 0, 0], [1, 1, 1], 0.15, 2)
    build_s = time.perf_counter() - t0
    kw = dict(flux="rusanov", cfl=0.3, final_time=1e9)
    s0 = H.initial_state("inner_cube", mesh, H.make_params(3, **kw))
    dm = H.DeviceMesh(mesh)
    out = {}
    res = {}
    for form in ("fp64", "mixed"):
        p = H.make_params(3, precision=form, **kw)
        ds, sv = H.DeviceState(3, mesh.num_cells), None
        sv = H.Solver(dm, p)
        ds.upload(s0, stream)
        sv.reset(0.0, stream)
        if form == "mixed" and shape:
            blk, cpt, sch = (int(v) for v in shape.split(","))
            sv.set_shape(blk, cpt, sch)
            out["mixed_launch_shape"] = {"block": blk, "cells_per_thread": cpt,
                                         "schedule": sch, "fixed": True}
        elif form == "mixed":
            out["mixed_launch_shape"] = sv.autotune(ds, 3, stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sv.run(ds, steps, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        code, t, _ = sv.status(stream)
        if code != 0:
            raise RuntimeError(f"3d {form}: status {code}")
        res[form] = ds.download(stream)
        out[form] = {"value": mesh.num_cells * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                     "t_final": t, "roofline": roofline_3d(mesh, form, sv.profile(ds, 4, stream),
                                                           ms / steps)}
        del sv, ds
    f, m = res["fp64"], res["mixed"]
    E = lambda s: s[0] * (s[4] + 0.5 * (s[1] ** 2 + s[2] ** 2 + s[3] ** 2))
    rel = lambda a, b: float(np.abs(a - b).sum() / np.abs(b).sum())
    out.update({"cells": mesh.num_cells, "faces": mesh.num_faces, "steps": steps,
                "host_mesh_build_s": build_s,
                "l1_density": rel(m[0], f[0]), "linf_density": float(np.abs(m[0] - f[0]).max()),
                "l1_total_energy": rel(E(m), E(f)), "linf_total_energy": float(np.abs(E(m) - E(f)).max()),
                "config": f"{n}^3 hex on [0,1]^3 jittered +-0.15h (seed 2), inner cube, Rusanov, "
                          f"CFL 0.3, walls, {steps} steps"})
    return out


def timed_steps(torch, solver, dstate, stream, K, dist):
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.run(dstate, K, stream=stream)  # fvh_solver_run: the time loop of driver.h:317-413
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if dist:
        ms = max_over_ranks(dist, ms)
        dist.barrier()
    return ms


def e2e_steps(solver, dstate, host, steps, warmup, stream, dist) -> float:
    """Seconds for `steps` calls of fvh_solver_advance_host, one step each,
    pinned host state in and out (max over ranks)."""
    t_sim = 0.0
    for _ in range(warmup):
        t_sim = solver.advance_host(dstate, host, 1, t_sim, stream)
    if dist:
        dist.barrier()
    w0 = time.perf_counter()
    for _ in range(steps):
        t_sim = solver.advance_host(dstate, host, 1, t_sim, stream)
    return max_over_ranks(dist, time.perf_counter() - w0)


def run_ours(args):
    import torch
    dist, ws, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    H, mesh, p64, p32, state0 = build_problem(args.n)
    stream = torch.cuda.Stream()
    dmesh = H.DeviceMesh(mesh)
    nc = mesh.num_cells
    results, finals, shape = {}, {}, None
    host = torch.empty((7, nc), dtype=torch.float64, pin_memory=True).numpy()
    with ClockSampler(local) as clk:
        for form, params in (("fp64", p64), ("mixed", p32)):
            dstate = H.DeviceState(2, nc)
            solver = H.Solver(dmesh, params)
            dstate.upload(state0, stream)
            solver.reset(0.0, stream)
            if form == "mixed" and args.shape:
                blk, cpt, sch = (int(v) for v in args.shape.split(","))
                solver.set_shape(blk, cpt, sch)
                shape = {"block": blk, "cells_per_thread": cpt, "schedule": sch, "fixed": True}
            elif form == "mixed":
                shape = solver.autotune(dstate, 5, stream)
            for _ in range(args.warmup):
                solver.step(dstate, stream)
            ms = timed_steps(torch, solver, dstate, stream, args.steps, dist)
            code, t, cell = solver.status(stream)
            if code != 0:
                raise RuntimeError(f"{form}: device status {code} at cell {cell}")
            finals[form] = dstate.download(stream)
            # end to end through the C ABI from pinned host memory, same workload
            host[:] = state0[:7]
            e2e_s = e2e_steps(solver, dstate, host, args.steps, args.warmup, stream, dist)
            results[form] = {"ms": ms, "launches": solver.launches_per_run(args.steps), "t": t,
                             "solver": solver, "state": dstate, "e2e_s": e2e_s}
    clocks = clk.summary()

    # per-kernel timings (CUDA events between launches on the stream)
    prof = {f: results[f]["solver"].profile(results[f]["state"], 10, stream) for f in results}

    # The rate after the configured 200 steps of the workload: the waves have
    # then spread over more of the mesh, and the kernels skip less work on
    # cells whose neighbourhood is uniform (their products with zero
    # differences and gradients).
    late = {}
    for form in results:
        sv, ds = results[form]["solver"], results[form]["state"]
        ds.upload(state0, stream)
        sv.reset(0.0, stream)
        sv.run(ds, 200, stream=stream)
        late[form] = timed_steps(torch, sv, ds, stream, args.steps, dist)
        if sv.status(stream)[0] != 0:
            raise RuntimeError(f"{form}: device status after 200 steps")

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    hbm, peak_kind = peaks()
    traffic, pipes = ncu_traffic(), ncu_pipes()

    def roofline(form):
        """Dominant kernel of the form: algorithmic bytes per launch over its
        duration.  The per-kernel event times of fvh_solver_profile are taken
        with an event between every two launches, which serialises the step
        a little; each kernel's duration here is its profiled share of the
        in-run step time (ms_per_step of the timed run)."""
        ab = algorithmic_bytes(mesh, form)
        p = prof[form]
        if "face_colour" in p:  # one launch per colour: the stage's bytes over its launches
            ab["face_colour"] = ab["face_colour_stage"] / (p["face_colour"][1] / 2)
        profiled_step = sum(v[0] * v[1] for v in p.values())
        in_run_step = results[form]["ms"] / args.steps
        scale = in_run_step / profiled_step
        dom = max(p, key=lambda k: p[k][0] * p[k][1])
        dur = p[dom][0] * scale
        achieved = ab[dom] / (dur * 1e-3) / 1e9
        tr = traffic.get(f"{form}:{dom}", {})
        out = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
               "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_kind,
               "traffic": tr.get("bytes"), "traffic_commit": tr.get("commit"),
               "algorithmic_bytes_per_launch": ab[dom],
               "duration_ms": dur,
               "duration_note": "profiled per-kernel event time x (in-run ms_per_step / "
                                f"profiled step {profiled_step:.4f} ms = {scale:.3f})",
               "kernels": {k: {"duration_ms": v[0] * scale, "launches_per_step": v[1],
                               "share": v[0] * v[1] / profiled_step,
                               "achieved_gbs": ab[k] / (v[0] * scale * 1e-3) / 1e9,
                               "frac": ab[k] / (v[0] * scale * 1e-3) / 1e9 / hbm,
                               "fp64_pipe_active": pipes.get(f"{form}:{k}", {}).get("fp64"),
                               "alu_pipe_active": pipes.get(f"{form}:{k}", {}).get("alu"),
                               "dram_traffic": traffic.get(f"{form}:{k}", {}).get("bytes")}
                           for k, v in p.items()}}
        if form == "mixed" and dom in ("gradients", "pack_dt"):
            # The per-task bytes of the reference dataflow (FP64 values, int32
            # connectivity), the same per-cell figure as the plain form's, for
            # comparability between forms; the kernel's own minimum (FP32
            # records) beside it.
            task = {"gradients": "gradients", "pack_dt": "dt"}[dom]
            sb = algorithmic_bytes(mesh, "fp64")[task]
            out.update({"algorithmic_bytes_per_launch": sb,
                        "achieved": sb / (dur * 1e-3) / 1e9,
                        "frac": sb / (dur * 1e-3) / 1e9 / hbm,
                        "bytes_basis": f"reference-dataflow bytes of the {task} task "
                                       f"({sb / mesh.num_cells:.0f} B/cell, as for the plain form)",
                        "kernel_bytes_per_launch": ab[dom],
                        "achieved_kernel_bytes": achieved,
                        "frac_kernel_bytes": achieved / hbm})
        return out

    zu = lambda ms: ws * nc * args.steps / (ms * 1e-3)
    m, f = finals["mixed"], finals["fp64"]
    l1 = lambda a, b: float(np.abs(a - b).sum() / np.abs(b).sum())
    E = lambda s: s[0] * (s[3] + 0.5 * (s[1] ** 2 + s[2] ** 2))

    def e2e(form):
        # the step reads d, v, e, p, a from the host planes and writes all 7
        bi, bo = 6 * 8 * nc, 7 * 8 * nc
        first = "dt" if form == "fp64" else "pack_dt"
        call = (f"fvh_solver_advance_host (pinned host state in, 1 step, host state out; the "
                f"first kernel ({first}) reads and the last update writes the host planes "
                "directly)")
        return {"value": ws * nc * args.steps / results[form]["e2e_s"], "unit": UNIT,
                "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo, "call": call}

    fp64_roof = roofline("fp64")
    fp64_roof["pipe_bound"] = "fp64"
    fp64_roof["note"] = ("the bit-exact FP64 kernels are bound by GB300's FP64 pipe (2 FP64 "
                         "operations per clock per SM) and by the integer pipe that computes "
                         "their products and quotients; fp64_pipe_active / alu_pipe_active per "
                         "kernel are the ncu figures (profiles/pipe_utilization.json)")
    line = {
        "metric": METRIC,
        "value": zu(results["fp64"]["ms"]),
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": results["fp64"]["ms"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(mesh),
        "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
        "algorithmic_bytes_per_zone_update": per_zone_update_bytes(mesh, "fp64"),
        "clocks": clocks,
        "e2e": e2e("fp64"),
        "gpu_launches": results["fp64"]["launches"],
        "after_200_steps": {"value": zu(late["fp64"]),
                            "ms_per_step": late["fp64"] / args.steps,
                            "note": f"{args.steps} steps timed after the configured 200 steps "
                                    "of the workload (less of the mesh is uniform then)"},
        "roofline": fp64_roof,
        "mixed": {"value": zu(results["mixed"]["ms"]),
                  "ms_per_step": results["mixed"]["ms"] / args.steps,
                  "dtype": "f32+f64",
                  "form": "FP32 reconstruction + Riemann flux, compensated FP32 face sums, "
                          "double-float increments onto the FP64 state, FP64 dt",
                  "gpu_launches": results["mixed"]["launches"],
                  "launch_shape": shape,
                  "after_200_steps": {"value": zu(late["mixed"]),
                                      "ms_per_step": late["mixed"] / args.steps},
                  "algorithmic_bytes_per_zone_update": per_zone_update_bytes(mesh, "mixed"),
                  "e2e": e2e("mixed"),
                  "roofline": roofline("mixed")},
        "mixed_over_fp64": results["fp64"]["ms"] / results["mixed"]["ms"],
        "accuracy": {"steps": args.warmup + args.steps,
                     "l1_density_mixed_vs_fp64": l1(m[0], f[0]),
                     "l1_total_energy_mixed_vs_fp64": l1(E(m), E(f)),
                     "linf_density_mixed_vs_fp64": float(np.abs(m[0] - f[0]).max()),
                     "linf_total_energy_mixed_vs_fp64": float(np.abs(E(m) - E(f)).max())},
        "conservation": {"note": "FP64 totals; outflow boundaries, so they change by the "
                                 "boundary fluxes",
                         "initial": conservation_totals(mesh, state0),
                         "fp64": conservation_totals(mesh, f),
                         "mixed": conservation_totals(mesh, m)},
    }
    for form in ("fp64", "mixed"):
        results[form]["solver"].close()
        del results[form]["state"]
    if not args.no_batch:
        line["batched"] = run_batched(torch, stream, min(args.steps, 50), args.warmup)
        line["batched_over_fp64"] = line["batched"]["value"] / line["value"]
        if args.serve_seconds > 0:
            line["serving"] = run_serving(torch, stream, line["batched"]["value"],
                                          args.serve_seconds)
    if not args.no_3d:
        line["shock_box_3d"] = run_3d(torch, stream, args.n3d, args.steps3d)
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.n)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_only_2d(args):
    """One form of the 2D workload alone: warm-up steps, then the timed steps
    in one fvh_solver_run (fixed launch shape for the mixed form if --shape)."""
    import torch
    torch.cuda.set_device(0)
    H, mesh, p64, p32, state0 = build_problem(args.n)
    stream = torch.cuda.Stream()
    params = p64 if args.only_2d == "fp64" else p32
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
    solver = H.Solver(dmesh, params)
    dstate.upload(state0, stream)
    solver.reset(0.0, stream)
    if args.only_2d == "mixed" and args.shape:
        solver.set_shape(*(int(v) for v in args.shape.split(",")))
    for _ in range(args.warmup):
        solver.step(dstate, stream)
    ms = timed_steps(torch, solver, dstate, stream, args.steps, None)
    code, t, cell = solver.status(stream)
    if code != 0:
        raise RuntimeError(f"{args.only_2d}: device status {code} at cell {cell}")
    print(json.dumps({"form": args.only_2d, "cells": mesh.num_cells, "steps": args.steps,
                      "ms_per_step": ms / args.steps,
                      "value": mesh.num_cells * args.steps / (ms * 1e-3)}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 512-problem batched form")
    ap.add_argument("--shape", default="",
                    help="fixed mixed launch shape 'block,cells_per_thread,schedule' "
                         "instead of autotuning (profiling runs)")
    ap.add_argument("--no-3d", action="store_true",
                    help="skip the 3D shock box (192^3, FP64 vs mixed, 100 steps)")
    ap.add_argument("--n3d", type=int, default=192, help="3D shock box side (default 192)")
    ap.add_argument("--steps3d", type=int, default=100, help="3D shock box steps (default 100)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the serving run (0 skips it)")
    ap.add_argument("--n", type=int, default=N_SIDE, help="mesh side (default 1024)")
    ap.add_argument("--only-2d", choices=["fp64", "mixed"], default="",
                    help="run only one form of the 2D workload (warm-up + steps) and print its "
                         "time (profiling of that form's kernels)")
    ap.add_argument("--only-3d", type=int, default=0, metavar="N",
                    help="run only the 3D shock box on an N^3 mesh for --steps steps and print "
                         "its record (profiling of the 3D kernels)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.only_3d:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(run_3d(torch, torch.cuda.Stream(), args.only_3d, args.steps,
                                args.shape)), flush=True)
        return 0
    if args.only_2d:
        return run_only_2d(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
