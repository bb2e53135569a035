"""Trigger pairs on the GPU (psx_world_trigger_events) against the oracle.

The GPU world and the oracle run in lockstep (the oracle fed the GPU's contact order),
so both follow the same trajectory; each frame's enter and exit events must then be the
same set.  The oracle's events equal the reference's callbacks
(tests/test_oracle_triggers.py)."""
import os
import sys

import numpy as np
import pytest

from physecs_gb300 import scenes
from tests.parity import gpu_keys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _scene_events(ev, scene):
    """GPU events of one scene as (frame, kind, body0, collider0, body1, collider1)."""
    sel = ev[:, 2] == scene
    return make_golden.events_sorted(ev[sel][:, [0, 1, 3, 4, 5, 6]])


def _lockstep_events(ss, frames, drain_every=1, **world_kw):
    """Steps a GPU world and one oracle per scene in lockstep; returns the GPU events and
    each oracle's events, drained every `drain_every` frames."""
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    g = World(ss, **world_kw)
    os_ = [OracleScene(s) for s in ss]
    got, want = [], [[] for _ in ss]
    for f in range(frames):
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        for i, o in enumerate(os_):
            sel = ids[:, 0] == i
            o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
            o.step()
            assert o.order_error() == 0
        if (f + 1) % drain_every == 0 or f + 1 == frames:
            ev, lost = g.trigger_events(cap=64)
            assert lost == 0
            got.append(ev)
            for i, o in enumerate(os_):
                want[i].append(o.trigger_events())
    assert g.counts()["error"] == 0
    got = np.concatenate(got)
    return g, got, [make_golden.events_sorted(np.concatenate(w)) for w in want]


@pytest.mark.parametrize("name", list(make_golden.trigger_scenes()))
def test_trigger_events_match_oracle(gpu_lib, oracle_lib, name):
    s, frames = make_golden.trigger_scenes()[name]
    _, got, (want,) = _lockstep_events([s], frames)
    assert len(want) > 50
    assert np.array_equal(_scene_events(got, 0), want)
    # delivery order: by frame, enter before exit
    order = got[:, 0] * 2 + got[:, 1]
    assert (np.diff(order) >= 0).all()


def test_trigger_events_in_a_batched_world_with_a_graph(gpu_lib, oracle_lib):
    """Trigger scenes beside a scene without triggers, frames replayed from the CUDA graph,
    events drained every 7 frames: each scene's events are its own oracle's."""
    sc = make_golden.trigger_scenes()
    ss = [sc["zones_a"][0], scenes.batch_scene(7, n_bodies=60), sc["flagged"][0], sc["zones_b"][0]]
    g, got, want = _lockstep_events(ss, 60, drain_every=7, use_graph=True)
    assert not (got[:, 2] == 1).any()
    for i in (0, 2, 3):
        assert len(want[i]) > 20
        assert np.array_equal(_scene_events(got, i), want[i]), i
    # entities are the scenes' own entity ids
    for e in got[:50]:
        st = ss[int(e[2])].arrays
        assert e[7] == st["entity"][e[3]] and e[8] == st["entity"][e[5]]


class _Recorder:
    def __init__(self, log, tag):
        self.log, self.tag = log, tag

    def on_trigger_enter(self, e0, c0, e1, c1):
        self.log.append((self.tag, 0, e0, c0, e1, c1))

    def on_trigger_exit(self, e0, c0, e1, c1):
        self.log.append((self.tag, 1, e0, c0, e1, c1))


def test_trigger_listeners(gpu_lib):
    """Listeners registered per scene run in registration order, each entering pair calling
    every enter listener, then the exits (src/Physecs.cpp:537-552); a removed listener no
    longer runs; a small drain capacity delivers the same events in the same order."""
    from physecs_gb300.api import World
    s, _ = make_golden.trigger_scenes()["zones_b"]
    w = World([s, s])
    log = []
    a, b, c = _Recorder(log, "a"), _Recorder(log, "b"), _Recorder(log, "c")
    w.add_on_trigger_enter_callback(a)
    w.add_on_trigger_enter_callback(b)
    w.add_on_trigger_exit_callback(a)
    w.add_on_trigger_enter_callback(c, scene=1)
    w.step(frames=40)
    ev = w.dispatch_trigger_events()
    ev0 = ev[ev[:, 2] == 0]
    assert len(ev0) > 20 and (ev0[:, 1] == 1).any()
    want = []
    for f, kind, _sc, _b0, c0, _b1, c1, e0, e1 in ev0.tolist():
        for tag in (("a", "b") if kind == 0 else ("a",)):
            want.append((tag, kind, e0, c0, e1, c1))
    assert [x for x in log if x[0] != "c"] == want
    assert len([x for x in log if x[0] == "c"]) == int(((ev[:, 2] == 1) & (ev[:, 1] == 0)).sum())
    w.remove_on_trigger_enter_callback(b)
    with pytest.raises(ValueError):
        w.remove_on_trigger_enter_callback(b)
    log.clear()
    w.step(frames=40)
    ev = w.dispatch_trigger_events()
    assert not any(x[0] == "b" for x in log)
    # the same 40 frames in a fresh world, drained 5 events at a time
    w2 = World([s, s])
    w2.step(frames=80)
    parts = []
    while True:
        e, lost = w2.trigger_events(cap=5)
        assert lost == 0
        parts.append(e)
        if len(e) == 0:
            break
    allev = np.concatenate(parts)
    assert np.array_equal(allev[allev[:, 0] >= 40], ev)


def test_world_without_triggers(gpu_lib):
    from physecs_gb300.api import World
    w = World([scenes.batch_scene(7, n_bodies=60)])
    w.step(frames=10)
    ev, lost = w.trigger_events()
    assert len(ev) == 0 and lost == 0
