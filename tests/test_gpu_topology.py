"""Topology changes between frames on the GPU, against the oracle.

Bodies destroyed and created (registry.destroy / registry.create with EnTT's entity
recycling), colliders cleared and added (Scene::clearColliders / addCollider) and joints
destroyed and created (Scene::destroyJoint / createJoint) between frames: the oracle edits
its scene in place, the device gets a world rebuilt by psx_world_recreate with the
continued colliders' bounds, restitution cache and trigger pairs and the joints' colours
and gear angles carried over (tests/topology_mirror.py keeps the description).  Every
frame in lockstep with the oracle fed the GPU's contact order: live bodies' state within
1e-5 relative.  The oracle is pinned to the reference on the same edits
(tests/test_oracle_topology.py, tests/golden/topology.npz)."""
import os
import sys

import numpy as np
import pytest

from tests.parity import gpu_keys, rel_state_diff

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from topology_mirror import SceneMirror  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _lockstep(s, frames, edit, use_graph=True):
    """edit(f, oracle, mirror) -> True when it changed the topology before frame f."""
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    g = World([s], use_graph=use_graph)
    o = OracleScene(s)
    m = SceneMirror(s)
    dead = set()
    edits = 0
    for f in range(frames):
        if edit(f, o, m, dead):
            g.synchronize()
            ns, carry = m.build(g.read_bodies())
            g.recreate([ns], [carry])
            edits += 1
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0, "frame %d: GPU manifolds not found in the oracle" % f
        st, so = g.read_bodies(), o.state()
        live = np.array([b not in dead for b in range(len(so["pos"]))])
        d = rel_state_diff({k: v[live] for k, v in st.items()}, {k: v[live] for k, v in so.items()})
        assert d <= TOL, "frame %d: relative state difference %g" % (f + 1, d)
    assert g.counts()["error"] == 0
    g.close()
    return edits


def test_entities_destroyed_and_created(gpu_lib, oracle_lib):
    s, sch, frames, _ = make_golden.topology_case()

    def edit(f, o, m, dead):
        if f not in sch:
            return False
        kill, spawn = sch[f]
        for b in kill:
            o.destroy_body(b)
            m.destroy_body(b)
            dead.add(b)
        for sp in spawn:
            b, e = o.create_body(sp)
            assert m.create_body(sp, e) == b
        return True
    assert _lockstep(s, frames, edit) == len(sch)


def test_joints_destroyed_and_created(gpu_lib, oracle_lib):
    s, plan, fr, frames = make_golden.joint_topology_case()

    def edit(f, o, m, dead):
        if f not in plan:
            return False
        kind, arg = plan[f]
        if kind == "destroy":
            o.destroy_joint(arg)
            m.destroy_joint(arg)
        else:
            assert o.create_joint(arg[0], arg[1], arg[2], fr) == m.create_joint(arg[0], arg[1], arg[2], fr)
        return True
    assert _lockstep(s, frames, edit) == len(plan)


def test_colliders_cleared_and_added(gpu_lib, oracle_lib):
    s, plan, frames = make_golden.collider_topology_case()

    def edit(f, o, m, dead):
        if f not in plan:
            return False
        for act in plan[f]:
            if act[0] == "clear":
                o.clear_colliders(act[1])
                m.clear_colliders(act[1])
            else:
                o.add_collider(act[1], act[2])
                m.add_collider(act[1], act[2])
        return True
    assert _lockstep(s, frames, edit, use_graph=False) == len(plan)


def test_trigger_pairs_carry_across_a_recreate(gpu_lib, oracle_lib):
    """A trigger scene whose bodies are destroyed and created: the trigger pairs of the
    frame before each change carry over, so no pair enters twice, and the events equal
    the oracle's frame by frame."""
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    from scene_variants import spawn_body, trigger_scene
    s = trigger_scene(41)
    a = s.arrays
    trig = [b for b in range(5, 95) if a["col_is_trigger"][a["collider_start"][b]]]
    rng = np.random.default_rng(2)
    g, o, m = World([s]), OracleScene(s), SceneMirror(s)
    got = []
    for f in range(60):
        ch = False
        if f in (20, 40):
            b = trig.pop(0)
            o.destroy_body(b)
            m.destroy_body(b)
            ch = True
        if f in (30, 50):
            sp = spawn_body(rng, [0.0, 7.0, 0.0])
            sp.arrays["col_is_trigger"][:] = 1
            b, e = o.create_body(sp)
            assert m.create_body(sp, e) == b
            ch = True
        if ch:
            g.synchronize()
            ns, carry = m.build(g.read_bodies())
            g.recreate([ns], [carry])
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        ev, lost = g.trigger_events()
        assert lost == 0
        got.append(ev)
    # compare (frame, kind, entity0, collider0, entity1, collider1): a destroyed body's pairs
    # exit under its entity, which the device reports with body -1
    ents = np.array([B["entity"] for B in m.bodies], np.int64)
    ow = o.trigger_events()
    want = make_golden.events_sorted(np.stack([ow[:, 0], ow[:, 1], ents[ow[:, 2]], ow[:, 3], ents[ow[:, 4]], ow[:, 5]], 1))
    ge = np.concatenate([e for e in got if len(e)]) if any(len(e) for e in got) else np.zeros((0, 9), np.int64)
    assert any(e[3] < 0 or e[5] < 0 for e in ge)   # pairs of destroyed bodies exited
    ge = np.stack([ge[:, 0], ge[:, 1], ge[:, 7], ge[:, 4], ge[:, 8], ge[:, 6]], 1)
    assert len(want) > 50 and (ow[:, 2] >= 0).all()
    assert np.array_equal(make_golden.events_sorted(ge), want)
