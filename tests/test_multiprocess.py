"""Multi-rank logic of bench.py on CPU: world size 2 over gloo.

Every GPU runs an independent replica (the single-mesh step is not sharded);
bench.py takes the maximum elapsed time over ranks with an all-reduce and
reports all ranks' zone-updates over it.  Here each rank runs a small replica
on the oracle (CPU), the aggregation goes through the same helper, and both
ranks must agree with a direct computation.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    import flecsale_gb300.hydro as H
    import oracle
    from tests import _util as U
    d, ws, r, _ = bench.dist_setup("gloo")
    assert (ws, r) == (world, rank)
    mesh = H.HostMesh.box(2, (40, 30), [0, 0], [1, 1], 0.2, 1)
    p = H.make_params(2, flux="hllc", cfl=0.4, boundary="outflow")
    s = H.initial_state("four_quadrant", mesh, p)
    import time
    t0 = time.perf_counter()
    U.oracle_run(oracle.load(), mesh, s, p, 3 + rank)  # ranks take different times
    ms = (time.perf_counter() - t0) * 1e3
    ms_max = bench.max_over_ranks(d, ms, device="cpu")
    value = ws * mesh.num_cells * 3 / (ms_max * 1e-3)
    q.put((rank, ms, ms_max, value))
    dist.destroy_process_group()


def test_replicas_max_over_ranks_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    true_max = max(r[1] for r in res)
    assert all(abs(r[2] - true_max) < 1e-9 for r in res)
    assert res[0][3] == res[1][3]
