"""The replica path of `bench.py --gpus N` (one graph does not shard, every rank
decomposes its own copy): ranks join a gloo group, a barrier brackets the
timed region, the reported time is the maximum over ranks, and the reference
arm runs on rank 0 only.  Run as two CPU processes (world size 2)."""
import json
import multiprocessing as mp
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    import oracle
    from oracle import gen
    w, r, local, dist = bench.dist_setup()
    # each replica decomposes its own graph (the CPU oracle stands in for the
    # device here) and reports its own time; the job time is the slowest rank's
    s, d = gen.er(2000, 12000, seed=100 + r)
    rp, col = oracle.csr_dedup(2000, s, d)
    core, kmax = oracle.bz(rp, col)
    ok = oracle.check_local(rp, col, core) == 0
    bench.barrier(dist)
    t = bench.allmax(dist, 5.0 + 3.0 * r)
    bench.barrier(dist)

    class Args:
        steps, warmup, gpus = 1, 0, world
    rc = bench.run_reference(Args, bench.WORKLOADS["er65536"], w, r, dist) if r == 1 else 0
    q.put((r, w, local, t, ok, rc))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == o[0] for o in out)
    assert all(o[3] == 8.0 for o in out)  # max over ranks, seen by every rank
    assert all(o[4] for o in out)
    assert out[1][5] == 0  # the reference arm does no work on rank 1


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local, dist = bench.dist_setup()
    assert (w, r, local, dist) == (1, 0, 0, None)
    assert bench.allmax(None, 3.5) == 3.5
    assert json.loads(json.dumps({"x": np.float64(1.0).item()}))["x"] == 1.0
