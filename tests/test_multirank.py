"""Scene shards over several ranks, on CPU (gloo, world size 2).

The batched workload splits over ranks by body count (physecs_gb300.shard.partition)
with no data-path collective: the only cross-rank traffic is the timing barrier and
the max / sum reductions.  Each rank simulates its share with the oracle (standing in
for its GPU), and every scene's result equals that scene simulated by one process
alone, so the shard count does not change a result."""
import hashlib
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FRAMES = 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _digest(o):
    st = o.state()
    return hashlib.sha256(b"".join(st[k].tobytes() for k in ("pos", "quat", "vel", "ang_vel"))).hexdigest()


def _rank_main(rank, world, port, n_per_rank, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from oracle.port_api import OracleScene
    r, w, local = bench.dist_info()
    d = bench.Dist(w, local)
    d.barrier()
    mx = d.max(float(10 + rank))
    sm = d.sum(float(1 + rank))
    ss, cfg = bench.build_workload("batched", r, n_per_rank, None, w)
    res = {}
    for s in ss:
        o = OracleScene(s)
        o.step(frames=FRAMES)
        res[s.name] = (_digest(o), s.n_dynamic)
        o.close()
    d.barrier()
    d.close()
    out.put((r, w, mx, sm, res, cfg.get("workload")))


def test_partition_is_balanced_deterministic_and_complete():
    from physecs_gb300 import scenes
    from physecs_gb300.shard import partition
    wts = [scenes.batch_scene_bodies(i) for i in range(4096)]
    for n in (1, 2, 3, 8):
        parts = partition(wts, n)
        assert parts == partition(wts, n)
        assert sorted(i for p in parts for i in p) == list(range(4096))
        loads = [sum(wts[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(wts), loads
    assert partition([5, 1, 1, 1, 1, 1], 2) == [[0], [1, 2, 3, 4, 5]]


def test_router_balances_work_and_is_deterministic():
    from physecs_gb300.shard import Router
    rng = np.random.default_rng(1)
    work = rng.integers(8, 8192, 500) * rng.integers(1, 121, 500)
    a, b = Router(4), Router(4)
    ra = [a.route(int(x)) for x in work]
    assert ra == [b.route(int(x)) for x in work]
    assert max(a.load) - min(a.load) <= int(work.max())
    assert sorted(set(ra)) == [0, 1, 2, 3]


@pytest.mark.timeout(300)
def test_two_rank_shards_give_the_single_process_results():
    sys.path.insert(0, ROOT)
    import bench
    from oracle.port_api import OracleScene
    n_per_rank = 4
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, n_per_rank, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=240) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, w0, mx0, sm0, s0, wl0), (r1, w1, mx1, sm1, s1, wl1) = res
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert mx0 == mx1 == 11.0
    assert sm0 == sm1 == 3.0
    assert wl0 == wl1
    assert not set(s0) & set(s1), "ranks must simulate different scenes"
    # together the ranks hold the whole 2 x n_per_rank-scene workload, split by bodies
    ss, _ = bench.build_workload("batched", 0, 2 * n_per_rank, None, 1)
    assert set(s0) | set(s1) == {s.name for s in ss}
    b0 = sum(v[1] for v in s0.values())
    b1 = sum(v[1] for v in s1.values())
    assert abs(b0 - b1) <= max(s.n_dynamic for s in ss)
    # every scene's frames equal the scene simulated alone in this process
    for s in ss:
        o = OracleScene(s)
        o.step(frames=FRAMES)
        got = s0.get(s.name) or s1.get(s.name)
        assert got[0] == _digest(o), s.name
        o.close()
