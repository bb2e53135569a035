"""Serving form on the GPU: continuous batching of scene requests.

A request's result equals the result of a world holding that scene alone, bit for
bit, whatever slot it lands in, whatever else is in flight, and after a slot has
been used by an earlier request (the plain world path itself is checked against
the oracle in test_gpu_parity)."""
import numpy as np
import pytest

from physecs_gb300 import scenes

pytestmark = pytest.mark.gpu

CLASSES = [(64, 4), (256, 4), (1024, 2)]


def _pool():
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(5, 1 << 19)), count=8)
    s = scenes.SceneData("pool")
    s.convex.extend(pool)
    s.add_bodies(pos=[[0, 0, 0]], quat=[scenes.IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3),
                 inv_inertia=np.zeros(9), col_type=scenes.SPHERE, col_params=[0.5, 0, 0, 0], col_mesh=-1)
    return pool, s.finalize()


def _requests(pool, ids, n_bodies):
    return [scenes.batch_scene(i, n_bodies=n, config=5, chain_prob=0.0, pool=pool) for i, n in zip(ids, n_bodies)]


def _alone(scene, frames):
    from physecs_gb300.api import World
    w = World([scene])
    w.step(frames=frames)
    w.synchronize()
    return w.read_bodies()


def _same(a, b):
    for k in ("pos", "quat", "vel", "ang_vel"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_request_alone_equals_mixed(gpu_lib):
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    reqs = _requests(pool, [11, 12, 13, 14, 15], [40, 200, 9, 700, 120])
    frames = [12, 7, 20, 9, 15]
    srv = Server(CLASSES, mesh_pool=pool_scene)
    live = {}
    results = {}
    t = 0
    # staggered admissions: request i arrives at tick 2*i
    pending = list(range(len(reqs)))
    while pending or live:
        while pending and 2 * pending[0] <= t:
            i = pending.pop(0)
            slot = srv.admit(reqs[i], frames[i])
            assert slot is not None
            live[slot] = i
        for slot in srv.tick():
            results[live.pop(slot)] = srv.read(slot)
            srv.release(slot)
        t += 1
        assert t < 200
    for i, r in enumerate(reqs):
        _same(results[i], _alone(r, frames[i]))


def test_slot_reuse_starts_clean(gpu_lib):
    """A request placed in a slot that another request just left sees none of its state
    (bodies, dynamic entries, cached contacts)."""
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    a, b = _requests(pool, [21, 22], [60, 60])
    srv = Server([(64, 1)], mesh_pool=pool_scene)
    sa = srv.admit(a, 5)
    while not srv.tick():
        pass
    srv.release(sa)
    sb = srv.admit(b, 6)
    assert sb == sa
    done = []
    while not done:
        done = srv.tick()
    _same(srv.read(sb), _alone(b, 6))


def test_admission_limits(gpu_lib):
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    small, big = _requests(pool, [31, 32], [30, 300])
    import ctypes as C
    from physecs_gb300.api import load
    from physecs_gb300.desc import make_desc
    srv = Server([(64, 1)], mesh_pool=pool_scene)
    lib = load()

    def admit_c(scene):
        slot = C.c_int32(-1)
        d = make_desc(scene)
        return lib.psx_server_admit(srv.h, C.byref(d), 3, C.c_float(1 / 60), C.byref(slot))

    assert admit_c(big) == 3                  # larger than the largest class: PSX_ERR_CAPACITY
    assert b"largest slot class" in lib.psx_last_error_string()
    assert srv.admit(big, 3) is None
    s0 = srv.admit(small, 3)
    assert s0 is not None
    assert admit_c(small) == 3                # no free slot
    assert srv.admit(small, 3) is None
    st = srv.stats()
    assert st["running"] == 1 and st["free"] == 0 and st["slots"] == 1


def test_pipelined_ticks_admit_while_a_frame_runs(gpu_lib):
    """Admissions, reads and releases between tick_begin and tick_end: requests admitted
    while a frame is in flight start with the next frame, and every result still equals
    the scene simulated alone."""
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    reqs = _requests(pool, [41, 42, 43, 44], [35, 150, 300, 12])
    frames = [6, 9, 4, 11]
    srv = Server(CLASSES, mesh_pool=pool_scene)
    live, results, pending = {}, {}, list(range(len(reqs)))
    slot = srv.admit(reqs[0], frames[0])
    live[slot] = 0
    pending.pop(0)
    srv.tick_begin()
    finished = []
    for t in range(40):
        for sl in finished:                  # the finished requests are read beside the frame in flight
            results[live.pop(sl)] = srv.read(sl)
            srv.release(sl)
        finished = []
        if pending and t % 2 == 0:           # admitted while a frame runs
            i = pending.pop(0)
            live[srv.admit(reqs[i], frames[i])] = i
        finished = srv.tick_end()
        if not live and not pending:
            break
        srv.tick_begin()
    for sl in finished:
        results[live.pop(sl)] = srv.read(sl)
        srv.release(sl)
    assert not live
    for i, r in enumerate(reqs):
        _same(results[i], _alone(r, frames[i]))


def test_profiled_ticks_report_stages_and_keep_results(gpu_lib):
    """A server made with profile=True times each tick's stages with CUDA events; its
    results are those of the graph-replaying server."""
    from physecs_gb300.api import Server
    pool, ps = _pool()
    reqs = _requests(pool, [41, 42], [200, 700])
    frames = 5
    out = []
    for profile in (False, True):
        srv = Server(CLASSES, mesh_pool=ps, profile=profile)
        slots = [srv.admit(s, frames) for s in reqs]
        stages = []
        for _ in range(frames):
            srv.tick()
            if profile:
                stages.append(srv.tick_stages())
        out.append([srv.read(sl) for sl in slots])
        srv.close()
    for a, b in zip(*out):
        _same(a, b)
    st = np.array(stages)
    assert st.shape == (frames, 6) and (st >= 0).all()
    assert (st[:, 1:5].sum(axis=1) > 0).all()
    assert st[0, 0] > 0   # the first tick uploads the admitted requests


def test_hbm_budget_caps_the_slots(gpu_lib):
    """Every slot keeps its request's state resident in device memory, so the HBM budget
    caps the slots a server may create; the server reports what it holds."""
    from physecs_gb300.api import PsxError, Server
    pool, pool_scene = _pool()
    srv = Server(CLASSES, mesh_pool=pool_scene)
    need = srv.device_bytes()
    srv.close()
    assert need > 0
    with pytest.raises(PsxError, match="OUT_OF_MEMORY"):
        Server(CLASSES, mesh_pool=pool_scene, hbm_budget=need // 2)
    srv = Server(CLASSES, mesh_pool=pool_scene, hbm_budget=need)
    assert srv.device_bytes() == need
    reqs = _requests(pool, [51], [100])
    slot = srv.admit(reqs[0], 2)
    srv.tick(); srv.tick()
    _same(srv.read(slot), _alone(reqs[0], 2))
    srv.close()


def _trigger_requests(pool, ids, n_bodies):
    """Serving requests with about one collider in eight a trigger (never the ground):
    dynamic triggers fall through the other bodies, so pairs enter and exit."""
    reqs = _requests(pool, ids, n_bodies)
    for i, s in zip(ids, reqs):
        a = s.arrays
        ncol = len(a["col_type"])
        cols = np.random.default_rng(i).permutation(np.arange(1, ncol))
        a["col_is_trigger"][cols[: max(1, ncol // 8)]] = 1
    return reqs


def _alone_events(scene, frames):
    from physecs_gb300.api import World
    w = World([scene])
    w.step(frames=frames)
    ev, lost = w.trigger_events()
    assert lost == 0
    w.close()
    return ev


def _request_events(ev, slot):
    got = ev[ev[:, 2] == slot].copy()
    got[:, 2] = 0
    return got


def test_trigger_events_per_request_equal_alone(gpu_lib):
    """Each request's trigger events, served beside others and in slots that earlier
    requests left the tick before, equal those of its scene stepped alone: same frames
    (counted from the request's first), bodies, colliders, entities and order."""
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    reqs = _trigger_requests(pool, [61, 62, 63, 64, 65, 66], [40, 200, 50, 180, 30, 60])
    frames = [25, 18, 30, 12, 22, 16]
    srv = Server([(64, 2), (256, 1)], mesh_pool=pool_scene, triggers=True)
    pending, live = list(range(len(reqs))), {}
    got = {i: [] for i in range(len(reqs))}

    def admit_waiting():
        for i in list(pending):
            slot = srv.admit(reqs[i], frames[i])
            if slot is not None:
                live[slot] = i
                pending.remove(i)

    admit_waiting()
    for _ in range(200):
        done = srv.tick()
        ev, lost = srv.trigger_events(cap=64)
        assert lost == 0
        for slot, i in live.items():
            got[i].append(_request_events(ev, slot))
        for slot in done:                    # released and refilled before the next tick
            live.pop(slot)
            srv.release(slot)
        admit_waiting()
        if not live and not pending:
            break
    assert not live and not pending
    total = exits = 0
    for i, r in enumerate(reqs):
        want = _alone_events(r, frames[i])
        have = np.concatenate(got[i])
        assert np.array_equal(have, want), i
        total += len(want)
        exits += int((want[:, 1] == 1).sum())
    assert total > 0 and exits > 0
    srv.close()


def test_trigger_events_of_a_request_released_mid_tick(gpu_lib):
    """A running request released while its tick is in flight, and a new request admitted
    into the same slot at once: the old request's events of that tick are decoded with its
    own bodies, the new one's start clean."""
    from physecs_gb300.api import Server
    pool, pool_scene = _pool()
    a, b = _trigger_requests(pool, [71, 72], [50, 60])
    srv = Server([(64, 1)], mesh_pool=pool_scene, triggers=True)
    sa = srv.admit(a, 40)
    ran = 14
    events = []
    for _ in range(ran - 1):
        assert not srv.tick()
        events.append(srv.trigger_events()[0])
    srv.tick_begin()                         # frame ran - 1 of a in flight
    srv.release(sa)
    sb = srv.admit(b, 9)
    assert sb == sa
    assert srv.tick_end() == []
    events.append(srv.trigger_events()[0])
    assert np.array_equal(_request_events(np.concatenate(events), sa), _alone_events(a, ran))
    events = []
    done = []
    while not done:
        done = srv.tick()
        events.append(srv.trigger_events()[0])
    assert np.array_equal(_request_events(np.concatenate(events), sb), _alone_events(b, 9))
    srv.close()
