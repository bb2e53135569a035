"""Registry deltas in the CPU oracle (a patched pose and its bounds, written velocities,
Scene::setIsKinematic; src/Physecs.cpp:51-54, 78-90, 753-770) against the reference:
body states of scenes stepped with seeded deltas between frames, recorded from the
reference (tests/golden/deltas.npz, tests/golden/make_golden.py), and the reference
itself side by side where its library is built."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from scene_variants import delta_schedule  # noqa: E402


@pytest.mark.parametrize("name", list(make_golden.delta_scenes()))
def test_oracle_deltas_match_reference_fixture(oracle_lib, name):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import pack_deltas
    d = np.load(os.path.join(HERE, "golden", "deltas.npz"))
    s, frames, rec = make_golden.delta_scenes()[name]
    pre = name + "__"
    assert str(d[pre + "scene_sha256"]) == make_golden.scene_hash(s)
    sch = delta_schedule(s, frames)
    o = OracleScene(s)
    for f in range(frames):
        if f in sch:
            o.apply_deltas(pack_deltas(sch[f]))
        o.step()
        if f + 1 in rec:
            for k, v in o.state().items():
                assert np.array_equal(v.view(np.uint32), d[pre + "f%d_%s" % (f + 1, k)].view(np.uint32)), (f + 1, k)


def test_pack_deltas_fold_order(oracle_lib):
    """Within one batch a kinematic toggle zeroes the velocities written before it; a
    velocity written after it stays."""
    from oracle.port_api import OracleScene
    from physecs_gb300 import scenes
    from physecs_gb300.api import pack_deltas
    s = scenes.batch_scene(3, n_bodies=20)
    b = int(np.nonzero(s.arrays["flags"] & scenes.BODY_DYNAMIC)[0][0])
    o = OracleScene(s)
    o.apply_deltas(pack_deltas([{"body": b, "vel": [1, 2, 3]}, {"body": b, "kinematic": True}]))
    assert (o.state()["vel"][b] == 0).all()
    o.apply_deltas(pack_deltas([{"body": b, "kinematic": False}, {"body": b, "vel": [1, 2, 3]}]))
    assert list(o.state()["vel"][b]) == [1, 2, 3]


def test_oracle_deltas_match_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    from physecs_gb300 import scenes
    from physecs_gb300.api import pack_deltas
    for s in (scenes.batch_scene(44, n_bodies=70, chain_prob=1.0), scenes.joint_chains(n_chains=3, links=5, seed=9)):
        sch = delta_schedule(s, 30, seed=17, every=2)
        o, r = OracleScene(s), RefScene(s)
        for f in range(30):
            if f in sch:
                d = pack_deltas(sch[f])
                o.apply_deltas(d)
                r.apply_deltas(d)
            o.step()
            r.step()
        so, sr = o.state(), r.state()
        for k in so:
            assert np.array_equal(so[k].view(np.uint32), sr[k].view(np.uint32)), (s.name, k)
