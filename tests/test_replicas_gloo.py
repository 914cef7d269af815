"""Multi-GPU mode is replicas only: every rank solves its own system with no
data-path collective; the benchmark takes the max time over ranks.  The
aggregation (process group, barrier, max-reduce) runs here as world-size-2
gloo ranks on CPU, each rank solving a small system with the CPU oracle."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), RSCHOL_BENCH_BACKEND="gloo")
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import rank_structured_cholesky_gb300 as rs
    from oracle import pyoracle as po
    r, w, dist = bench.dist_setup(world)
    prob = rs.diffusion(2, 24 + 8 * r, sigma=1.0, seed=r)   # each replica its own system
    F = po.OracleFactor(prob.colptr, prob.rowind, prob.vals, prob.xyz, dict(max_dense_block=8, max_diag_block=32))
    assert F.factor() == 0
    _, it, _, res = F.pcg(prob.rhs[0], 1e-8, 500)
    bench.barrier(dist)
    t = bench.reduce_max(dist, float(10 + r), "cpu")
    out.put((r, w, it, res, t))
    dist.destroy_process_group()


def test_two_replicas_max_reduce():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [2, 2]
    assert all(r[4] == 11.0 for r in res)           # max over ranks
    assert all(r[3] <= 1e-8 for r in res)
