"""Trigger pairs of the CPU oracle (Scene::simulate's trigger set and its onTriggerEnter /
onTriggerExit callbacks, src/Physecs.cpp:200-207, 537-552) against the reference: the
golden callbacks in tests/golden/triggers.npz, recorded from the reference's own
listeners (tests/golden/make_golden.py), and, where the reference library is built,
fresh scenes side by side."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
from scene_variants import trigger_scene  # noqa: E402

FIX = os.path.join(HERE, "golden", "triggers.npz")


@pytest.mark.parametrize("name", list(make_golden.trigger_scenes()))
def test_oracle_trigger_events_match_reference_fixture(oracle_lib, name):
    from oracle.port_api import OracleScene
    d = np.load(FIX)
    s, frames = make_golden.trigger_scenes()[name]
    pre = name + "__"
    assert str(d[pre + "scene_sha256"]) == make_golden.scene_hash(s)
    o = OracleScene(s)
    for _ in range(frames):
        o.step()
    got = make_golden.events_sorted(o.trigger_events())
    want = d[pre + "events"]
    assert len(want) > 50 and set(want[:, 1]) == {0, 1}
    assert np.array_equal(got, want)
    assert len(o.trigger_events()) == 0   # drained


def test_trigger_event_semantics():
    """Per pair, enter and exit alternate and start with an enter; an enter and an exit of
    the same pair never fall in one frame; every event pair has a trigger collider."""
    d = np.load(FIX)
    s, _ = make_golden.trigger_scenes()["zones_b"]
    trig = s.arrays["col_is_trigger"]
    cs = s.arrays["collider_start"]
    last = {}
    for f, kind, b0, c0, b1, c1 in d["zones_b__events"].tolist():
        assert trig[cs[b0] + c0] or trig[cs[b1] + c1]
        key = (b0, c0, b1, c1)
        prev = last.get(key)
        assert (prev is None and kind == 0) or (prev is not None and prev[1] != kind and prev[0] < f)
        last[key] = (f, kind)
    # a jointed pair with a trigger raises events (the trigger test comes before the filter)
    jb = set(zip(s.arrays["joint_body0"].tolist(), s.arrays["joint_body1"].tolist()))
    jointed = [e for e in d["zones_b__events"].tolist() if (e[2], e[4]) in jb or (e[4], e[2]) in jb]
    assert jointed


def test_scene_without_triggers_raises_no_events(oracle_lib):
    from oracle.port_api import OracleScene
    from physecs_gb300 import scenes
    o = OracleScene(scenes.batch_scene(7, n_bodies=60))
    for _ in range(20):
        o.step()
    assert len(o.trigger_events()) == 0


def test_oracle_trigger_events_match_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    for seed in (43, 44):
        s = trigger_scene(seed, n=60)
        o, r = OracleScene(s), RefScene(s)
        for k in range(80):
            o.step()
            r.step()
            if k % 20 == 19:   # drained every 20 frames, as a caller between frames would
                assert np.array_equal(make_golden.events_sorted(o.trigger_events()),
                                      make_golden.events_sorted(r.trigger_events())), (seed, k)
