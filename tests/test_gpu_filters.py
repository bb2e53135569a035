"""A user contact filter and setCanCollide on the GPU (psx_world_set_contact_filter,
psx_world_set_can_collide) against the oracle, in lockstep (the oracle fed the GPU's
contact order): states bit for bit every frame and the same trigger events, with the
frame replayed from a CUDA graph that each change makes the world capture again.  The
oracle's filters equal the reference's (tests/test_oracle_filters.py)."""
import os
import sys

import numpy as np
import pytest

from tests.parity import gpu_keys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def test_filters_match_oracle(gpu_lib, oracle_lib):
    from oracle.port_api import OracleScene
    from physecs_gb300 import scenes
    from physecs_gb300.api import World
    s, filt, cc, frames, _ = make_golden.filter_case()
    plain = scenes.batch_scene(5, n_bodies=40)
    g = World([plain, s], use_graph=True)
    o = OracleScene(s)
    g.set_contact_filter(filt)
    o.set_contact_filter(filt)
    got = []
    for f in range(frames):
        if f in cc:
            g.set_can_collide(*cc[f], scene=1)
            o.set_can_collide(*cc[f])
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        sel = ids[:, 0] == 1
        o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
        o.step()
        assert o.order_error() == 0
        st, so = g.read_bodies(), o.state()
        sl = slice(g.body_start[1], g.body_start[2])
        for k in so:
            assert np.array_equal(st[k][sl].view(np.uint32), so[k].view(np.uint32)), (f, k)
        ev, lost = g.trigger_events()
        assert lost == 0
        got.append(ev)
    ev = np.concatenate(got)
    want = make_golden.events_sorted(o.trigger_events())
    assert len(want) > 100
    assert np.array_equal(make_golden.events_sorted(ev[ev[:, 2] == 1][:, [0, 1, 3, 4, 5, 6]]), want)
    # the filter applies to every scene: the plain scene's data are all 0, so it is unchanged
    assert g.counts()["error"] == 0


def test_default_filter_restored(gpu_lib):
    from physecs_gb300 import scenes
    from physecs_gb300.api import PsxError, World
    s = scenes.batch_scene(5, n_bodies=40)
    a, b = World([s]), World([s])
    a.set_contact_filter(lambda t0, d0, t1, d1: 1)     # every pair a trigger pair: bodies fall through
    a.step(frames=5)
    a.set_contact_filter(None)
    b.step(frames=5)
    assert not np.array_equal(a.read_bodies()["pos"], b.read_bodies()["pos"])
    with pytest.raises(PsxError):
        a.set_contact_filter(lambda t0, d0, t1, d1: 7)
