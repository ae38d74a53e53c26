"""Multi-GPU layout is replicas only: every rank applies the operator to its own
function, no collective touches the data path; the benchmark combines per-rank
results with a max over ranks (time) and a sum (node-terms).  This runs the
same helpers as bench.py with two gloo ranks on the CPU, each rank doing a CPU
oracle apply on its own seeded input."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bench
    import mrcpp_gb300 as mw
    import oracle
    from cases import gaussian_sum, project

    r, w, local, pg = bench.dist_setup(world)
    mra = mw.MRA(box=(-20, 20), order=3, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-2)
    f = project(mra, 1e-2, gaussian_sum(100 + r, 2, (2.0, 10.0), (-1.0, 1.0), (0.5, 1.0)))
    res = oracle.apply(1e-2, mw.FunctionTree(mra), P, f, nthreads=1)
    t = 1.0 + r  # a stand-in per-rank time
    tmax = bench.reduce_max(pg, t)
    nt = bench.reduce_sum(pg, res["node_terms"])
    bench.barrier(pg)
    q.put((r, res["node_terms"], tmax, nt))
    dist.destroy_process_group()


def test_two_rank_replica_reduction():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=300) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    total = out[0][1] + out[1][1]
    for r, own, tmax, nt in out:
        assert tmax == 2.0
        assert nt == total
