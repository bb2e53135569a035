"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

Each rank simulates its own scenes (weak scaling, no data-path collective); the
only cross-rank traffic is the timing barrier and the max / sum reductions."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_info()
    d = bench.Dist(w, local)
    d.barrier()
    mx = d.max(float(10 + rank))
    sm = d.sum(float(1 + rank))
    ss, cfg = bench.build_workload("batched", r, 3)
    first_seed = ss[0].arrays["pos"].tobytes()
    d.barrier()
    d.close()
    out.put((r, w, mx, sm, len(ss), first_seed, cfg.get("workload")))


@pytest.mark.timeout(300)
def test_two_rank_barrier_reductions_and_sharding():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, w0, mx0, sm0, n0, s0, wl0), (r1, w1, mx1, sm1, n1, s1, wl1) = res
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert mx0 == mx1 == 11.0
    assert sm0 == sm1 == 3.0
    assert n0 == n1 == 3
    assert wl0 == wl1
    assert s0 != s1, "ranks must simulate different scenes"
