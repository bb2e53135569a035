"""The narrowphase's filters in the CPU oracle against the reference: a user contact
filter (Scene::setContactFilter, src/Physecs.cpp:200, 795-797) and setCanCollide
(src/Physecs.cpp:209, 788-793) toggled between frames.  States and trigger events
recorded from the reference (tests/golden/filters.npz, tests/golden/make_golden.py)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402


def test_oracle_filters_match_reference_fixture(oracle_lib):
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "filters.npz"))
    s, filt, cc, frames, rec = make_golden.filter_case()
    assert str(d["scene_sha256"]) == make_golden.scene_hash(s)
    o = OracleScene(s)
    o.set_contact_filter(filt)
    for f in range(frames):
        if f in cc:
            o.set_can_collide(*cc[f])
        o.step()
        if f + 1 in rec:
            for k, v in o.state().items():
                assert np.array_equal(v.view(np.uint32), d["f%d_%s" % (f + 1, k)].view(np.uint32)), (f + 1, k)
    ev = make_golden.events_sorted(o.trigger_events())
    assert len(ev) > 100 and np.array_equal(ev, d["events"])


def test_filter_changes_the_outcome(oracle_lib):
    """The fixture's filter is not the default one: without it the same scene differs."""
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "filters.npz"))
    s, _, cc, frames, rec = make_golden.filter_case()
    o = OracleScene(s)
    for f in range(20):
        if f in cc:
            o.set_can_collide(*cc[f])
        o.step()
    assert not np.array_equal(o.state()["pos"], d["f20_pos"])
