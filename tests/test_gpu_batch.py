"""Batched form (fvh_batch_*): independent meshes advanced together.

A problem's cells only read cells of the same problem and its dt is the
maximum over its own cells, so every comparison here is bitwise: a problem in a
mix equals the same problem alone, whatever the launch shape, and equals the
single-mesh mixed solver.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H

pytestmark = pytest.mark.gpu

KINDS = ("kelvin_helmholtz", "four_quadrant", "sod")


def _problems(n, seed=3, lo=12, hi=72):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.integers(lo, hi))
        ny = int(rng.integers(lo, hi))
        mesh = H.HostMesh.box(2, (nx, ny), [0, 0], [1, 1], 0.2, 100 + k)
        kind = KINDS[k % len(KINDS)]
        out.append((mesh, kind))
    return out


def _params():
    return H.make_params(2, flux="hllc", precision="mixed", boundary="outflow", cfl=0.4,
                         final_time=10.0)


def _run_batch(problems, nsteps, tf=None, shape=None, bad=None):
    p = _params()
    meshes = [m for m, _ in problems]
    b = H.Batch.for_meshes(p, meshes)
    tfs = tf if tf is not None else [10.0] * len(meshes)
    b.assign(meshes, 0.4, tfs)
    if shape:
        b.set_shape(*shape)
    for k, (m, kind) in enumerate(problems):
        s = H.initial_state(kind, m, p, seed=k)
        if bad is not None and k == bad[0]:
            s[3, bad[1]] = -1.0
        b.set_state(k, s, 0.0)
    b.step(nsteps)
    t, codes, cells = b.query()
    return [b.get_state(k) for k in range(len(meshes))], t, codes, cells


def test_same_alone_and_in_the_mix():
    probs = _problems(9)
    mix, t_mix, codes, _ = _run_batch(probs, 25)
    assert np.all(codes == 0)
    for k in (0, 4, 8):
        alone, t_alone, c1, _ = _run_batch([probs[k]], 25)
        assert c1[0] == 0 and t_alone[0] == t_mix[k]
        assert np.array_equal(alone[0], mix[k])


def test_matches_single_mesh_mixed_solver(cuda):
    probs = _problems(4, seed=7)
    mix, t_mix, _, _ = _run_batch(probs, 20)
    p = _params()
    for k, (m, kind) in enumerate(probs):
        dm, ds = H.DeviceMesh(m), H.DeviceState(2, m.num_cells)
        s = H.Solver(dm, p)
        ds.upload(H.initial_state(kind, m, p, seed=k))
        s.reset(0.0)
        s.run(ds, 20)
        out = ds.download()
        assert s.status()[1] == t_mix[k]
        assert np.array_equal(out, mix[k])


def test_launch_shape_does_not_change_results():
    probs = _problems(5, seed=11)
    a, ta, _, _ = _run_batch(probs, 15)
    for shape in ((256, 1), (128, 3), (256, 2), (128, 1, 1), (256, 2, 1)):
        b, tb, codes, _ = _run_batch(probs, 15, shape=shape)
        assert np.all(codes == 0) and np.array_equal(ta, tb)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_per_problem_final_time():
    probs = _problems(6, seed=5)
    tfs = [0.004, 0.01, 0.02, 0.05, 0.003, 0.5]
    states, t, codes, _ = _run_batch(probs, 400, tf=tfs)
    assert np.all(codes == 0)
    for k in range(5):
        assert abs(t[k] - tfs[k]) <= 1e-12 * tfs[k] + 1e-15
    # a finished problem stays unchanged: more steps give the same state
    states2, t2, _, _ = _run_batch(probs, 420, tf=tfs)
    for k in range(5):
        assert np.array_equal(states[k], states2[k]) and t2[k] == t[k]


def test_failure_is_isolated_to_its_problem():
    probs = _problems(5, seed=9)
    good, _, codes, _ = _run_batch(probs, 10)
    bad, _, codes_b, cells_b = _run_batch(probs, 10, bad=(2, 17))
    assert codes_b[2] == H.ERR_NEGATIVE_STATE and cells_b[2] == 17
    for k in (0, 1, 3, 4):
        assert codes_b[k] == 0 and np.array_equal(bad[k], good[k])


def test_reassign_keeps_running_problems(cuda):
    """Continuous batching: problems 1 and 3 continue in a new assignment that
    drops the others and admits a new one; their results equal an
    uninterrupted run."""
    probs = _problems(5, seed=13)
    ref, tref, _, _ = _run_batch(probs, 30)
    p = _params()
    meshes = [m for m, _ in probs]
    extra = _problems(1, seed=99)[0]
    b = H.Batch(p, 200000, 400000, 200000, 8)
    b.assign(meshes, 0.4, 10.0)
    for k, (m, kind) in enumerate(probs):
        b.set_state(k, H.initial_state(kind, m, p, seed=k), 0.0)
    b.step(12)
    b.assign([meshes[3], extra[0], meshes[1]], 0.4, 10.0, keep=[3, -1, 1])
    b.set_state(1, H.initial_state(extra[1], extra[0], p, seed=1), 0.0)
    b.step(18)
    t, codes, _ = b.query()
    assert np.all(codes == 0)
    assert t[0] == tref[3] and t[2] == tref[1]
    assert np.array_equal(b.get_state(0), ref[3]) and np.array_equal(b.get_state(2), ref[1])


def test_autotune_picks_a_shape_and_keeps_results(tmp_path, monkeypatch):
    monkeypatch.setenv("FVH_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    probs = _problems(6, seed=21)
    ref, tref, _, _ = _run_batch(probs, 12)
    p = _params()
    meshes = [m for m, _ in probs]
    b = H.Batch.for_meshes(p, meshes)
    b.assign(meshes, 0.4, 10.0)
    for k, (m, kind) in enumerate(probs):
        b.set_state(k, H.initial_state(kind, m, p, seed=k), 0.0)
    best = b.autotune(trial_steps=2, use_cache=False)
    assert best["block"] in (128, 256) and best["schedule"] in (0, 1) and best["ms_per_step"] > 0
    assert (tmp_path / "tune.txt").read_text().strip()
    cached = b.autotune(trial_steps=2, use_cache=True)
    assert {k: cached[k] for k in ("block", "cells_per_thread", "schedule")} == \
           {k: best[k] for k in ("block", "cells_per_thread", "schedule")}
    b.step(12)  # tuning restored the state: results equal an untuned run
    t, codes, _ = b.query()
    assert np.all(codes == 0) and np.array_equal(t, tref)
    for k in range(len(meshes)):
        assert np.array_equal(b.get_state(k), ref[k])


def test_steps_split_across_calls_bitwise():
    """Within one fvh_batch_step call each corrector prepares the next step's
    pack and per-problem CFL maxima; splitting the steps over several calls
    (each starting from the FP64 state) must give the same bits."""
    probs = _problems(6, seed=21)
    tfs = [10.0, 0.01, 10.0, 0.02, 10.0, 10.0]
    one, t1, c1, _ = _run_batch(probs, 24, tf=tfs)
    p = _params()
    meshes = [m for m, _ in probs]
    b = H.Batch.for_meshes(p, meshes)
    b.assign(meshes, 0.4, tfs)
    for k, (m, kind) in enumerate(probs):
        b.set_state(k, H.initial_state(kind, m, p, seed=k), 0.0)
    for n in (5, 1, 7, 11):
        b.step(n)
    t2, c2, _ = b.query()
    assert np.all(c1 == 0) and np.all(c2 == 0) and np.array_equal(t1, t2)
    for k in range(len(meshes)):
        assert np.array_equal(b.get_state(k), one[k])


def test_mismatched_carried_problem_is_refused_and_changes_nothing():
    """A reassignment that carries a problem onto a mesh with a different cell
    count is refused with FVH_ERR_INVALID_ARGUMENT before anything on the
    device changes (host and device-side assignment): stepping on afterwards
    gives the same bits as a batch that never saw the bad call."""
    probs = _problems(3)
    p = _params()
    meshes = [m for m, _ in probs]

    def fresh():
        b = H.Batch.for_meshes(p, meshes, slack=2.0)
        b.assign(meshes, 0.4, 10.0)
        for k, (m, kind) in enumerate(probs):
            b.set_state(k, H.initial_state(kind, m, p, seed=k), 0.0)
        b.step(4)
        return b

    a, ref = fresh(), fresh()
    other = H.HostMesh.box(2, (7, 5), [0, 0], [1, 1], 0.2, 9)
    assert other.num_cells != meshes[0].num_cells
    with pytest.raises(H.FvhError) as ei:
        a.assign([other, meshes[1]], 0.4, 10.0, keep=[0, 1])
    assert ei.value.code == H.ERR_INVALID_ARGUMENT
    with pytest.raises(H.FvhError) as ei:
        H.batch_assign_device(a, [H.DeviceMesh(other), H.DeviceMesh(meshes[1])], 0.4, 10.0,
                              keep=[0, 1])
    assert ei.value.code == H.ERR_INVALID_ARGUMENT
    a.step(4)
    ref.step(4)
    ta, ca, _ = a.query()
    tr, cr, _ = ref.query()
    assert np.all(ca == 0) and np.array_equal(ta, tr)
    for k in range(len(meshes)):
        assert np.array_equal(a.get_state(k), ref.get_state(k))
