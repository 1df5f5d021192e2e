"""Continuous-batching solve server over the batched C ABI (fvh_batch_*).

Requests (a 2D problem of some size, kind and end time) arrive over time.  A
pool of host threads builds each request's mesh and uploads it to the device
once.  The server keeps every running request's state resident in one
fvh_batch and advances all of them together with one CUDA-graph launch of
`steps_per_launch` steps.  Between launches it drains finished requests
(downloading their state) and admits waiting ones whose meshes are on the
device and whose cells, faces and vertices fit in the batch's capacity; the
new set of problems is concatenated on the device (fvh_batch_assign_device),
and running requests keep their device state, so admissions and evictions
restart nobody and cost no host work proportional to the other requests.
Each request's result is the same as solving it alone (its cells only read its
own cells and its dt is a maximum over its own cells).

This module is the host driver; the step itself is libflecsale_gb300.so.
"""
from __future__ import annotations

import dataclasses
import time
from concurrent.futures import ThreadPoolExecutor
from typing import List, Optional

import numpy as np

from . import hydro as H


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    side: int               # side x side quad cells on [0,1]^2
    kind: str               # fvh_problem_kind name
    t_end: float
    seed: int = 0
    jitter: float = 0.2
    # filled by the server
    mesh: Optional[H.HostMesh] = None
    dmesh: Optional[H.DeviceMesh] = None
    state0: Optional[np.ndarray] = None
    admitted: float = -1.0
    finished: float = -1.0
    result: Optional[np.ndarray] = None
    t_final: float = 0.0
    status: int = 0


def poisson_requests(rate: float, duration: float, seed: int, side_range=(64, 2048),
                     t_end_range=(0.05, 0.3), kinds=("kelvin_helmholtz", "four_quadrant", "sod")):
    """Arrivals of a Poisson process of the given rate; sides log-uniform (so
    cells are log-uniform), end times uniform."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        side = int(round(np.exp(rng.uniform(np.log(side_range[0]), np.log(side_range[1])))))
        out.append(Request(rid=len(out), arrival=t, side=side, kind=kinds[len(out) % len(kinds)],
                           t_end=float(rng.uniform(*t_end_range)), seed=int(rng.integers(1 << 30))))


def server_params() -> H.Params:
    """Scheme of the batched/served forms: mixed precision, HLLC, transmissive
    boundaries, CFL 0.4, and textbook reconstruction (the reference's e/p
    gradient swap drives Sod negative before t = 0.3)."""
    return H.make_params(2, flux="hllc", precision="mixed", boundary="outflow", cfl=0.4,
                         swap=False, final_time=1.0e9)


def build_mesh(req: Request, params: Optional[H.Params] = None, upload: bool = False) -> Request:
    req.mesh = H.HostMesh.box(2, (req.side, req.side), [0, 0], [1, 1], req.jitter, req.seed)
    if params is not None:
        req.state0 = H.initial_state(req.kind, req.mesh, params, seed=req.seed)
    if upload:
        req.dmesh = H.DeviceMesh(req.mesh)
    return req


class Server:
    def __init__(self, params: H.Params, max_cells: int, max_faces: int, max_vertices: int,
                 max_problems: int = 512, steps_per_launch: int = 8, stream=None,
                 build_threads: int = 8):
        self.params = params
        self.batch = H.Batch(params, max_cells, max_faces, max_vertices, max_problems)
        self.caps = (max_cells, max_faces, max_vertices, max_problems)
        self.steps_per_launch = steps_per_launch
        self.stream = stream
        self.pool = ThreadPoolExecutor(build_threads)

    def _fits(self, running: List[Request], req: Request) -> bool:
        c = sum(r.mesh.num_cells for r in running) + req.mesh.num_cells
        f = sum(r.mesh.num_faces for r in running) + req.mesh.num_faces
        v = sum(r.mesh.num_vertices for r in running) + req.mesh.num_vertices
        return (c <= self.caps[0] and f <= self.caps[1] and v <= self.caps[2]
                and len(running) + 1 <= self.caps[3])

    def run(self, requests: List[Request], time_limit: float = 600.0) -> dict:
        b, p = self.batch, self.params
        pending = sorted(requests, key=lambda r: r.arrival)
        building, ready, running, done = [], [], [], []
        zone_updates = launches = reassigns = 0
        t0 = time.perf_counter()
        while pending or building or ready or running:
            now = time.perf_counter() - t0
            if now > time_limit:
                break
            while pending and pending[0].arrival <= now:
                building.append(self.pool.submit(build_mesh, pending.pop(0), p, True))
            still = []
            for fut in building:
                (ready.append(fut.result()) if fut.done() else still.append(fut))
            building = still
            # finished requests leave, waiting ones are admitted: one reassignment
            stay = list(range(len(running)))
            if running:
                times, codes, _ = b.query(self.stream)
                finished = [k for k, r in enumerate(running)
                            if codes[k] != 0 or times[k] >= r.t_end * (1 - 1e-12)]
                for k in finished:
                    r = running[k]
                    r.result = b.get_state(k, self.stream)
                    r.t_final, r.status = float(times[k]), int(codes[k])
                    r.finished = time.perf_counter() - t0
                    r.dmesh = None  # release its device copy
                    done.append(r)
                stay = [k for k in stay if k not in finished]
            kept = [running[k] for k in stay]
            admit = []
            for req in sorted(ready, key=lambda r: r.arrival):
                if self._fits(kept + admit, req):
                    admit.append(req)
            for req in admit:
                ready.remove(req)
            new = kept + admit
            if len(new) != len(running) or admit:
                if new:
                    H.batch_assign_device(b, [r.dmesh for r in new], p.cfl, [r.t_end for r in new],
                                          keep=stay + [-1] * len(admit), stream=self.stream)
                    for k, req in enumerate(admit, start=len(kept)):
                        b.set_state(k, req.state0, 0.0, self.stream)
                        req.admitted = time.perf_counter() - t0
                    reassigns += 1
                running = new
            if not running:
                time.sleep(0.001)  # idle until the next arrival or build completion
                continue
            b.step(self.steps_per_launch, self.stream)
            launches += 1
            zone_updates += sum(r.mesh.num_cells for r in running) * self.steps_per_launch
        wall = time.perf_counter() - t0
        tts = np.array([r.finished - r.arrival for r in done]) if done else np.zeros(0)
        return {
            "requests_done": len(done),
            "requests_total": len(requests),
            "wall_s": wall,
            "p50_time_to_solution_s": float(np.percentile(tts, 50)) if len(tts) else None,
            "p99_time_to_solution_s": float(np.percentile(tts, 99)) if len(tts) else None,
            "zone_updates": zone_updates,
            "zone_updates_per_s": zone_updates / wall,
            "graph_launches": launches,
            "reassignments": reassigns,
            "failed": sum(1 for r in done if r.status != 0),
            "done": done,
        }

    def close(self):
        self.pool.shutdown(wait=True)
        self.batch.close()


def fp64_rerun_l1(req: Request, params: H.Params) -> float:
    """Relative L1 density error of a served (mixed) result against the same
    request solved alone with the FP64 path to the same end time."""
    p64 = H.make_params(2, flux=_flux_name(params.flux_kind), precision="fp64",
                        boundary="outflow" if params.boundary == 1 else "wall",
                        swap=bool(params.recon_swap_ep), cfl=params.cfl, final_time=req.t_end)
    mesh = req.mesh or build_mesh(req).mesh
    dm, ds = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
    s = H.Solver(dm, p64)
    ds.upload(H.initial_state(req.kind, mesh, p64, seed=req.seed))
    s.reset(0.0)
    s.run(ds, 10**7, stop_at_final_time=True, check_every=64)
    ref = ds.download()
    return float(np.abs(req.result[0] - ref[0]).sum() / np.abs(ref[0]).sum())


def _flux_name(kind: int) -> str:
    return {v: k for k, v in H.FLUX.items()}[kind]
