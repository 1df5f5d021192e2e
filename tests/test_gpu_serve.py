"""Continuous-batching server (flecsale_gb300.serve) on small requests.

The device capacity is set so that only a few requests fit at once, so
requests queue, are admitted while others run, and leave at different times.
Each served result must equal the same request solved alone (bitwise: a batch
of one stepped to its end time), and stay within the mixed form's 1e-4
relative L1 density error of an FP64 rerun.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from flecsale_gb300 import serve


def _alone(req, p):
    r = serve.build_mesh(serve.Request(req.rid, 0.0, req.side, req.kind, req.t_end, req.seed))
    b = H.Batch.for_meshes(p, [r.mesh])
    b.assign([r.mesh], p.cfl, [r.t_end])
    b.set_state(0, H.initial_state(r.kind, r.mesh, p, seed=r.seed), 0.0)
    for _ in range(10000):
        b.step(5)
        t, codes, _ = b.query()
        if t[0] >= r.t_end * (1 - 1e-12) or codes[0] != 0:
            break
    return b.get_state(0), t[0]


@pytest.mark.gpu
def test_served_results_equal_solo_runs():
    p = serve.server_params()
    rng = np.random.default_rng(4)
    reqs = [serve.Request(rid=k, arrival=0.0, side=int(rng.integers(20, 64)),
                          kind=("kelvin_helmholtz", "four_quadrant", "sod")[k % 3],
                          t_end=float(rng.uniform(0.005, 0.03)), seed=k) for k in range(9)]
    srv = serve.Server(p, max_cells=3 * 64 * 64, max_faces=3 * 2 * 65 * 64,
                       max_vertices=3 * 65 * 65, max_problems=4, steps_per_launch=3)
    rep = srv.run(reqs, time_limit=120)
    srv.close()
    assert rep["requests_done"] == len(reqs) and rep["failed"] == 0
    assert rep["p99_time_to_solution_s"] >= rep["p50_time_to_solution_s"] > 0
    assert rep["reassignments"] >= 3
    assert any(r.admitted > min(q.finished for q in reqs) for r in reqs), \
        "capacity should have made some requests wait for others to finish"
    for r in reqs:
        solo, t_solo = _alone(r, p)
        assert r.t_final == t_solo
        assert np.array_equal(r.result, solo)
    for r in reqs[:4]:
        assert serve.fp64_rerun_l1(r, p) <= 1e-4


def test_poisson_request_stream():
    """Host-side request generator (no GPU)."""
    reqs = serve.poisson_requests(rate=5.0, duration=20.0, seed=4)
    assert 60 <= len(reqs) <= 140
    sides = np.array([r.side for r in reqs])
    assert sides.min() >= 64 and sides.max() <= 2048
    assert all(0.05 <= r.t_end <= 0.3 for r in reqs)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
