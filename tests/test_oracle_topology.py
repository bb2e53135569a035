"""Entities destroyed and created between frames in the CPU oracle, against the
reference: registry.destroy / registry.create with the reference's signal handlers
(onRigidBodyCreate / onRigidBodyDelete, onDynamicCreate / onDynamicDelete,
src/Physecs.cpp:25-66) and EnTT 3.12's storages (component storage swap-and-pop,
entity ids recycled most recent first with their version bumped).  Entity values and
states bit for bit: against tests/golden/topology.npz (made by the reference,
tests/golden/make_golden.py) and live where the reference library is built.  The
device path for topology changes is not built; this pins the semantics it must meet."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from scene_variants import topology_schedule  # noqa: E402


def _run(sim, sch, frames, rec=()):
    ents, states = [], {}
    for f in range(frames):
        if f in sch:
            kill, spawn = sch[f]
            for b in kill:
                sim.destroy_body(b)
            for sp in spawn:
                ents.append(sim.create_body(sp)[1])
        sim.step()
        if f + 1 in rec:
            states[f + 1] = sim.state()
    return ents, states


def test_oracle_topology_matches_reference_fixture(oracle_lib):
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "topology.npz"))
    s, sch, frames, rec = make_golden.topology_case()
    assert str(d["scene_sha256"]) == make_golden.scene_hash(s)
    ents, states = _run(OracleScene(s), sch, frames, rec)
    assert list(ents) == list(d["entities"])
    assert any(e >> 20 for e in ents) and any(not e >> 20 for e in ents)   # recycled and fresh ids
    for f in rec:
        for k, v in states[f].items():
            assert np.array_equal(v.view(np.uint32), d["f%d_%s" % (f, k)].view(np.uint32)), (f, k)


def test_oracle_topology_matches_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    from physecs_gb300 import scenes
    s = scenes.batch_scene(12, n_bodies=60, chain_prob=0.0)
    sch = topology_schedule(s, 40, seed=12, every=3)
    eo, so = _run(OracleScene(s), sch, 40, [40])
    er, sr = _run(RefScene(s), sch, 40, [40])
    assert eo == er
    for k in so[40]:
        assert np.array_equal(so[40][k].view(np.uint32), sr[40][k].view(np.uint32)), k


def test_oracle_joint_topology_matches_reference_fixture(oracle_lib):
    """Scene::createJoint / destroyJoint between frames (src/Physecs.cpp:690-725): a
    destroyed joint leaves its colour (the rest keep their order) and frees the colour
    and the pair; a new one takes the lowest colour free on both bodies."""
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "topology.npz"))
    s, plan, fr, frames = make_golden.joint_topology_case()
    assert str(d["joints_scene_sha256"]) == make_golden.scene_hash(s)
    st = make_golden.run_joint_plan(OracleScene(s), plan, fr, frames)
    for k, v in st.items():
        assert np.array_equal(v.view(np.uint32), d["joints_f%d_%s" % (frames, k)].view(np.uint32)), k


def test_oracle_collider_topology_matches_reference_fixture(oracle_lib):
    """Scene::addCollider / clearColliders between frames (src/Physecs.cpp:727-751): the
    new entry goes last with creation bounds; clearing swaps each entry out."""
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "topology.npz"))
    s, plan, frames = make_golden.collider_topology_case()
    assert str(d["colliders_scene_sha256"]) == make_golden.scene_hash(s)
    st = make_golden.run_collider_plan(OracleScene(s), plan, frames)
    for k, v in st.items():
        assert np.array_equal(v.view(np.uint32), d["colliders_f%d_%s" % (frames, k)].view(np.uint32)), k


def test_trigger_events_across_entity_changes_match_live_reference(oracle_lib):
    """Trigger bodies destroyed (their overlapping pairs exit) and trigger bodies created
    (their pairs enter) between frames give the reference's events."""
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    from scene_variants import spawn_body, trigger_scene
    s = trigger_scene(41)
    a = s.arrays
    trig = [b for b in range(5, 95) if a["col_is_trigger"][a["collider_start"][b]]]
    rng = np.random.default_rng(2)
    sims = [OracleScene(s), RefScene(s)]
    for f in range(80):
        if f in (20, 40):
            b = trig.pop(0)
            for sim in sims:
                sim.destroy_body(b)
        if f in (30, 50):
            sp = spawn_body(rng, [0.0, 7.0, 0.0])
            sp.arrays["col_is_trigger"][:] = 1
            for sim in sims:
                sim.create_body(sp)
        for sim in sims:
            sim.step()
    eo, er = (make_golden.events_sorted(sim.trigger_events()) for sim in sims)
    assert len(eo) > 100 and np.array_equal(eo, er)
    so, sr = sims[0].state(), sims[1].state()
    for k in so:
        assert np.array_equal(so[k].view(np.uint32), sr[k].view(np.uint32)), k
