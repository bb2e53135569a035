"""GPU parity: the CUDA path against the CPU oracle on the same seeded scenes.

Tolerances (from the hot path's parity contract):
  * collider bounds and broadphase pair sets: bit-exact;
  * manifold normals, points and target velocities from identical poses: 1e-5;
  * a frame from identical state, with the oracle fed the GPU's colour-sorted
    contact order: 1e-5 relative.
The library is built with -fmad=false, so in practice these match bit for bit.
"""
import numpy as np
import pytest

from physecs_gb300 import scenes
from tests.parity import compare_contacts, gpu_keys, pair_set, rel_state_diff
from tests.scene_variants import scattered_scene

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _mini_mixed(seed=7, n=60):
    return scenes.batch_scene(seed, n_bodies=n)


def _scenes():
    return {
        "pyramid": scenes.pyramid(rows=8),
        "mixed": _mini_mixed(),
        "chain": scenes.batch_scene(11, n_bodies=40, chain_prob=1.0),
        "heightfield": scenes.large_mixed(n_bodies=300, cells=32),
        "joints": scenes.joint_chains(n_chains=12, links=6),
        "scattered": scattered_scene(),
    }


@pytest.fixture(scope="module")
def all_scenes():
    return _scenes()


def _oracle(s):
    from oracle.port_api import OracleScene
    return OracleScene(s)


def _gpu(s, **kw):
    from physecs_gb300.api import World
    return World(s if isinstance(s, list) else [s], **kw)


@pytest.mark.parametrize("name", ["pyramid", "mixed", "chain", "heightfield", "joints", "scattered"])
def test_creation_bounds_bit_exact(all_scenes, name, gpu_lib, oracle_lib):
    s = all_scenes[name]
    g = _gpu(s)
    o = _oracle(s)
    gb = g.bounds()
    ids, ob = o.bounds()
    # oracle bounds are listed per collider in creation order before the first step
    starts = s.arrays["collider_start"]
    order = np.array([starts[e] + c for e, c in ids])
    assert np.array_equal(gb[order].view(np.uint32), ob.view(np.uint32))


@pytest.mark.parametrize("name", ["pyramid", "mixed", "chain", "heightfield", "joints", "scattered"])
def test_first_frame_pairs_and_manifolds(all_scenes, name, gpu_lib, oracle_lib):
    s = all_scenes[name]
    g = _gpu(s)
    o = _oracle(s)
    g.step(); g.synchronize()
    o.step()
    gp = g.pairs()[:, 1:]
    op = o.pairs()
    assert pair_set(gp) == pair_set(op)
    ids, gf, meta = g.contacts()
    _, of = o.contacts()
    worst = compare_contacts(gpu_keys(ids, meta), gf, o.contact_keys(), of)
    assert worst <= TOL, worst
    assert g.counts()["error"] == 0


@pytest.mark.parametrize("name,frames", [("pyramid", 40), ("mixed", 30), ("chain", 30), ("heightfield", 10), ("joints", 30)])
def test_frames_in_lockstep_with_oracle_fed_gpu_order(all_scenes, name, frames, gpu_lib, oracle_lib):
    """Each frame: step the GPU, hand its colour-sorted contact order to the oracle, step the
    oracle, compare full body state.  Any divergence shows up within a frame."""
    s = all_scenes[name]
    g = _gpu(s)
    o = _oracle(s)
    for f in range(frames):
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0, "frame %d: GPU manifolds not found in the oracle" % f
        d = rel_state_diff(g.read_bodies(), o.state())
        assert d <= TOL, "frame %d: relative state difference %g" % (f, d)
    assert g.counts()["error"] == 0


def test_batched_world_matches_scene_by_scene(gpu_lib, oracle_lib):
    """Eight uneven scenes in one world: every scene equals its own oracle run."""
    ss = [scenes.batch_scene(i, n_bodies=n) for i, n in enumerate([16, 40, 90, 23, 150, 64, 31, 200])]
    ss[3] = scenes.batch_scene(3, n_bodies=23, chain_prob=1.0)
    g = _gpu(ss)
    os_ = [_oracle(s) for s in ss]
    start = g.body_start
    for f in range(15):
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        st = g.read_bodies()
        for i, o in enumerate(os_):
            sel = ids[:, 0] == i
            o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
            o.step()
            assert o.order_error() == 0
            d = rel_state_diff({k: v[start[i]:start[i + 1]] for k, v in st.items()}, o.state())
            assert d <= TOL, "scene %d frame %d: %g" % (i, f, d)


def test_one_substep_from_identical_state(gpu_lib, oracle_lib):
    """One substep (substeps = 1) from an identical mid-simulation state."""
    s = scenes.pyramid(rows=10)
    o = _oracle(s)
    o.step(frames=25)
    st = o.state()
    s2 = scenes.pyramid(rows=10)
    s2.num_substeps = 1
    g = _gpu(s2)
    g.write_bodies(st)
    o.set_knobs(1, s.num_iterations, s.gravity)
    # same pose history matters only through the broadphase margins, which start fresh on both sides
    from oracle.port_api import OracleScene
    o2 = OracleScene(s2)
    o2.write_state(st)
    g.step(); g.synchronize()
    ids, gf, meta = g.contacts()
    o2.set_contact_order(gpu_keys(ids, meta))
    o2.step()
    assert o2.order_error() == 0
    assert rel_state_diff(g.read_bodies(), o2.state()) <= TOL


def _kat_scene_list(case):
    """The known-answer pair scenes of tests/golden/narrow_pairs.npz for one shape pair."""
    from tests.test_oracle_golden import SHAPES, _load, _meshes
    poses = _load("narrow_pairs.npz")[case + "__poses"]
    a, b = case.split("__")
    meshes = _meshes()
    ta, pa = SHAPES[a]
    out = []
    for p in poses:
        if b == "trimesh":
            out.append(scenes.pair_scene(ta, pa, (p[0:3], p[3:7]), scenes.TRIANGLE_MESH, [], ([0, 0, 0], scenes.IDENTITY_Q),
                                         mesh0=meshes.get(a), mesh1=meshes["trimesh"], dynamic=(True, False)))
        else:
            tb, pb = SHAPES[b]
            out.append(scenes.pair_scene(ta, pa, (p[0:3], p[3:7]), tb, pb, (p[7:10], p[10:14]),
                                         mesh0=meshes.get(a), mesh1=meshes.get(b)))
    return out


def test_narrowphase_every_shape_pair(gpu_lib, oracle_lib):
    """Every shape pair at the seeded touching poses of the known-answer fixtures, as one
    batched world per shape pair: GPU manifolds equal the oracle's (which equal the
    reference's, checked on the CPU)."""
    from tests.test_oracle_golden import _kat_cases
    for case in _kat_cases():
        ss = _kat_scene_list(case)
        g = _gpu(ss)
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        total = 0
        for i, s in enumerate(ss):
            o = _oracle(s)
            o.step()
            sel = ids[:, 0] == i
            _, of = o.contacts()
            worst = compare_contacts(gpu_keys(ids[sel], meta[sel]), gf[sel], o.contact_keys(), of)
            assert worst <= TOL, (case, i, worst)
            total += int(sel.sum())
        assert total > 0, case
        assert g.counts()["error"] == 0, case


def test_scene_results_independent_of_batch(gpu_lib):
    """A scene gives bit-identical results alone and at any position of any batch: its
    broadphase order, manifold order and contact colouring depend on the scene only.
    This is what lets a serving batch admit and retire requests freely."""
    a = scenes.batch_scene(5, n_bodies=150, chain_prob=1.0)
    others = [scenes.batch_scene(100 + i, n_bodies=n) for i, n in enumerate([40, 300, 17, 90])]
    runs = []
    for batch, pos in (([a], 0), ([others[0], others[1], a], 2), ([a] + others, 0), (others[:2] + [a] + others[2:], 2)):
        g = _gpu(batch)
        g.step(frames=30)
        g.synchronize()
        st = g.read_bodies()
        s0, s1 = g.body_start[pos], g.body_start[pos + 1]
        runs.append({k: v[s0:s1] for k, v in st.items()})
        assert g.counts()["error"] == 0
    for r in runs[1:]:
        for k in r:
            assert np.array_equal(r[k].view(np.uint32), runs[0][k].view(np.uint32)), k


def _plate_with_spheres(n_side=15):
    """A dynamic 16 x 16 m plate on the ground carrying n_side^2 spheres: the plate
    touches more bodies than the colour limit, so its contacts overflow into the
    serially solved last colour."""
    s = scenes.SceneData("plate")
    scenes._ground_box(s, (30.0, 0.5, 30.0))
    he = (8.0, 0.25, 8.0)
    m, com, I = scenes.mass_box(he)
    s.add_bodies(pos=[[0.0, 0.25, 0.0]], quat=[scenes.IDENTITY_Q], flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m,
                 com=com, inv_inertia=np.linalg.inv(I).T.ravel(), col_type=scenes.BOX, col_params=[*he, 0.0])
    r = 0.4
    ms, comS, IS = scenes.mass_sphere(r)
    g = (np.arange(n_side) - (n_side - 1) / 2.0) * 1.0
    xs, zs = np.meshgrid(g, g)
    pos = np.stack([xs.ravel(), np.full(xs.size, 0.5 + r - 0.005), zs.ravel()], axis=1)
    s.add_bodies(pos=pos, quat=np.tile(scenes.IDENTITY_Q, (len(pos), 1)), flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / ms,
                 com=comS, inv_inertia=np.linalg.inv(IS).T.ravel(), col_type=scenes.SPHERE, col_params=[r, 0, 0, 0])
    return s.finalize()


def test_contacts_beyond_the_colour_limit(gpu_lib, oracle_lib):
    """A body with more contacts than colours: the overflow colour is solved serially in
    contact order, and the frame still equals the oracle fed the GPU's order."""
    s = _plate_with_spheres()
    g = _gpu(s)
    o = _oracle(s)
    for f in range(4):
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        assert int(meta[:, 0].max()) + 1 == 128 or f > 0
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0
        assert rel_state_diff(g.read_bodies(), o.state()) <= TOL
    assert g.counts()["error"] == 0


def test_graph_launched_frames_equal_eager_frames(gpu_lib):
    """use_graph: the first frame runs eagerly, the second is captured, later ones replay
    the graph; the states equal those of eager frames bit for bit."""
    ss = [scenes.batch_scene(70 + i, n_bodies=n) for i, n in enumerate([30, 1200, 90])]
    a = _gpu(ss)
    b = _gpu(ss, use_graph=True)
    for f in range(6):
        a.step(); b.step()
        a.synchronize(); b.synchronize()
        sa, sb = a.read_bodies(), b.read_bodies()
        for k in sa:
            assert np.array_equal(sa[k].view(np.uint32), sb[k].view(np.uint32)), (f, k)
    assert b.counts()["kernels"] > 0


def test_kinematic_trigger_disabled_and_empty_scenes(gpu_lib, oracle_lib):
    """A ragged batch with kinematic bodies, trigger and disabled colliders, a scene without
    dynamic bodies and a scene without contacts: every scene equals its own oracle run."""
    from tests.scene_variants import apart_scene, flagged_scene, static_only_scene
    ss = [flagged_scene(), static_only_scene(), apart_scene(), scenes.pyramid(rows=3), flagged_scene(32, 40)]
    g = _gpu(ss)
    os_ = [_oracle(s) for s in ss]
    start = g.body_start
    for f in range(20):
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        st = g.read_bodies()
        gp = g.pairs()
        for i, o in enumerate(os_):
            sel = ids[:, 0] == i
            o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
            o.step()
            assert o.order_error() == 0
            if f == 0:
                assert pair_set(gp[gp[:, 0] == i][:, 1:]) == pair_set(o.pairs())
            d = rel_state_diff({k: v[start[i]:start[i + 1]] for k, v in st.items()}, o.state())
            assert d <= TOL, "scene %d frame %d: %g" % (i, f, d)
    assert g.counts()["error"] == 0


def test_capacity_overflow_is_reported(gpu_lib):
    """A pair capacity far below the scene's pair count: the frame reports
    PSX_ERR_CAPACITY through the device error word instead of dropping pairs silently."""
    from physecs_gb300.api import PsxError
    s = scenes.pyramid(rows=40)   # 820 cubes: about 2500 pairs once the margins apply
    g = _gpu(s, pairs_per_collider=1, manifolds_per_collider=1)   # capacity max(1024, colliders)
    g.step(frames=3)
    with pytest.raises(PsxError, match="CAPACITY"):
        g.synchronize()


def test_launch_shapes_do_not_change_results(gpu_lib):
    """Any launch configuration the tuner may pick gives the same frames bit for bit."""
    ss = [scenes.batch_scene(80 + i, n_bodies=n) for i, n in enumerate([60, 1300, 200, 25])]
    a = _gpu(ss)
    others = [_gpu(ss, launch=dict(convex_warps=3, convex_blocks_per_sm=5, analytic_threads=128, analytic_blocks_per_sm=4,
                                   contacts_threads=256, solver_smem_kb=100, gjk_blocks_per_sm=4, epa_lanes=32)),
              _gpu(ss, launch=dict(epa_lanes=16, convex_warps=1, convex_blocks_per_sm=4, large_threads=128)),
              _gpu(ss, launch=dict(epa_lanes=8, convex_warps=1, convex_blocks_per_sm=2, large_threads=256)),
              _gpu(ss, launch=dict(epa_full_only=1, solver_threads_min=256)),
              _gpu(ss, launch=dict(epa_lanes=1, convex_blocks_per_sm=8)),
              _gpu(ss, launch=dict(solver_threads_min=32))]
    assert [o.launch_config()["epa_lanes"] for o in others[:3]] == [32, 16, 8]
    assert others[4].launch_config()["epa_lanes"] == 1
    assert others[5].launch_config()["solver_threads_min"] == 32
    assert others[3].launch_config()["epa_full_only"] == 1 and others[3].launch_config()["solver_threads_min"] == 256
    for f in range(8):
        a.step()
        a.synchronize()
        sa = a.read_bodies()
        for b in others:
            b.step()
            b.synchronize()
            sb = b.read_bodies()
            for k in sa:
                assert np.array_equal(sa[k].view(np.uint32), sb[k].view(np.uint32)), (f, k, b.launch_config())
    b = others[0]
    cfg = b.tune(frames=1)
    assert set(cfg) >= {"convex_warps", "analytic_threads", "solver_smem_kb"}


@pytest.mark.parametrize("solver", [1, 2], ids=["cluster", "grid"])
@pytest.mark.parametrize("kind", ["mixed", "chains"])
def test_large_scene_on_a_cluster_or_the_grid(gpu_lib, oracle_lib, kind, solver):
    """Scenes above the 8192-body block limit are solved by a thread-block cluster (velocities
    in distributed shared memory) or by the whole grid; either way frames stay in lockstep
    with the oracle."""
    s = scenes.batch_scene(9, n_bodies=9000) if kind == "mixed" else scenes.joint_chains(n_chains=300, links=32)
    assert s.n_dynamic > 8192
    g = _gpu(s, launch={"large_scene_solver": solver})
    assert g.launch_config()["large_scene_solver"] == solver
    o = _oracle(s)
    for f in range(4):
        g.step(); g.synchronize()
        ids, gf, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0, f
        d = rel_state_diff(g.read_bodies(), o.state())
        assert d <= TOL, "frame %d: %g" % (f, d)
    assert g.counts()["error"] == 0


def _colouring(s, **kw):
    g = _gpu(s, **kw)
    g.step(); g.synchronize()
    ids, _, meta = g.contacts()
    key = np.concatenate([ids[:, 4:8], meta[:, 1:2]], axis=1)
    order = np.lexsort(key.T[::-1])
    return key[order], meta[order, 0], ids[order, 1:3]


def test_colouring_is_the_same_on_a_cluster_the_grid_and_a_block(gpu_lib):
    """The contact colouring depends only on the scene: a scene solved by a thread-block
    cluster or by the whole grid gets the colours it gets from a single block, and no
    colour holds two contacts of one dynamic body."""
    s = scenes.large_mixed(n_bodies=9000, cells=256)
    kc, cc, bc = _colouring(s, launch={"large_scene_solver": 1})
    kg, cg, _ = _colouring(s, launch={"large_scene_solver": 2})
    kb, cb, bb = _colouring(s, block_scene_max_dyn=1 << 30)
    assert np.array_equal(kc, kb) and np.array_equal(kg, kb)
    assert np.array_equal(cc, cb), "colour counts %s vs %s" % (np.bincount(cc[cc >= 0])[:16], np.bincount(cb[cb >= 0])[:16])
    assert np.array_equal(cg, cb)
    assert (cc >= 0).all() and cc.max() > 4
    for c in range(cc.max() + 1):
        sel = cc == c
        bodies = bc[sel].ravel()
        bodies = bodies[bodies >= 0]
        assert len(np.unique(bodies)) == len(bodies), "colour %d" % c


def test_body_io_through_pinned_and_pageable_arrays(gpu_lib):
    """read_bodies / write_bodies / simulate_host repack on the device: the same results
    from page-locked and from ordinary arrays, static bodies reading zero velocity, and a
    round trip that leaves the world as it was."""
    from physecs_gb300.api import World, pin_host, unpin_host
    s = scenes.batch_scene(21, n_bodies=120)
    a, b = World([s]), World([s])
    a.step(frames=3)
    b.step(frames=3)
    st = a.read_bodies()
    static = (s.arrays["flags"] & scenes.BODY_DYNAMIC) == 0
    assert (st["vel"][static] == 0).all() and (st["ang_vel"][static] == 0).all()
    a.write_bodies(st)
    pin_host(*st.values())
    try:
        a.simulate_host(s.dt, st)
    finally:
        unpin_host(*st.values())
    sb = b.read_bodies()
    b.simulate_host(s.dt, sb)
    for k in st:
        assert np.array_equal(st[k].view(np.uint32), sb[k].view(np.uint32)), k


def _hull_heavy(seed=5, n=400):
    """Mostly convex hulls in a pile that starts interpenetrating (about 1800 manifolds on the
    first frame, 180 by the twelfth): many overlapping convex pairs, shallow and deep."""
    rng = scenes.SplitMix64(scenes.scene_seed(12, seed))
    s = scenes.SceneData("hulls%d" % seed)
    scenes._ground_box(s, (8.0, 0.5, 8.0))
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(12, 1 << 19)), count=8)
    s.convex.extend(pool)
    centers = scenes._jittered_grid(rng, 8, 7, 8, 1.1, [0.0, 1.2, 0.0])[:n]
    scenes._mixed_bodies(s, rng, centers, 0, pool, mix=(0.1, 0.1, 0.2, 0.6))
    return s.finalize()


@pytest.mark.parametrize("lanes,full_only", [(1, 2), (1, 1), (8, 2), (16, 2), (16, 1), (32, 2)])
def test_epa_schedules_agree_with_the_oracle(lanes, full_only, gpu_lib, oracle_lib):
    """EPA with a lane per pair (new faces built by the whole warp; pairs needing more than
    12 steps handed to the grouped kernel, or with full_only 1 to the full polytope), and
    with 8, 16 or 32 lanes per pair (full_only 1: the full polytope alone): manifolds
    from identical poses within the contract (in practice bit for bit) on a hull pile,
    and the frames in lockstep with the oracle fed the GPU's contact order."""
    s = _hull_heavy()
    g = _gpu(s, launch=dict(epa_lanes=lanes, epa_full_only=full_only, convex_blocks_per_sm=8), pairs_per_collider=32,
             manifolds_per_collider=16)
    o = _oracle(s)
    for f in range(1, 13):
        g.step()
        g.synchronize()
        ids, gf, meta = g.contacts()
        keys = gpu_keys(ids, meta)
        o.set_contact_order(keys)
        o.step()
        assert o.order_error() == 0, "frame %d" % f
        _, of = o.contacts()
        worst = compare_contacts(keys, gf, o.contact_keys(), of)
        assert worst <= TOL, "frame %d: manifolds differ by %g" % (f, worst)
        d = rel_state_diff(g.read_bodies(), o.state())
        assert d <= TOL, "frame %d: relative state difference %g" % (f, d)
        nc = g.narrow_counts()
        assert nc["convex"] >= nc["epa"] >= max(nc["past_lane"], nc["past_group"]) and nc["past_group"] >= 0
        assert nc["epa"] > 0 and (nc["past_lane"] >= nc["past_group"] if lanes == 1 else nc["past_lane"] == 0)
        assert full_only == 2 or nc["past_group"] == 0
    assert g.counts()["error"] == 0


def _clustered_scene(seed=3):
    """576 spheres spread over a grid and one cluster of 60 overlapping spheres: the
    cluster's first leaves have far more partners than the average collider."""
    rng = np.random.default_rng(seed)
    s = scenes.SceneData("clustered")
    scenes._ground_box(s, (40.0, 0.5, 40.0))
    grid = np.array([[x, 2.0, z] for x in np.arange(-36.0, 36.0, 3.0) for z in np.arange(-36.0, 36.0, 3.0)])
    cluster = rng.uniform(-0.6, 0.6, size=(60, 3)) + [0.0, 4.0, 0.0]
    pos = np.concatenate([grid, cluster]).astype(np.float32)
    s.add_bodies(pos=pos, quat=[scenes.IDENTITY_Q] * len(pos), flags=scenes.BODY_DYNAMIC, inv_mass=1.0,
                 com=np.zeros(3), inv_inertia=np.eye(3).ravel(), col_type=scenes.SPHERE,
                 col_params=[0.4, 0.0, 0.0, 0.0], col_mesh=-1)
    return s.finalize()


def test_pairs_beyond_the_kept_ones_keep_their_order(gpu_lib, oracle_lib):
    """The walk keeps a leaf's first pairs (4.5 x pairs_per_collider of them) and walks
    again only for leaves with more.  With 4 pairs per collider the cluster's leaves take
    that second walk; the pair list, order included, is that of a world whose leaves all
    fit (64 pairs per collider), and the set is the oracle's."""
    s = _clustered_scene()
    tight, roomy = _gpu(s, pairs_per_collider=4), _gpu(s, pairs_per_collider=64)
    for f in range(3):
        for g in (tight, roomy):
            g.step(); g.synchronize()
        a, b = tight.pairs(), roomy.pairs()
        assert f > 0 or len(a) > 1000   # the cluster separates over the next frames
        assert np.array_equal(a, b), f
    o = _oracle(s)
    g = _gpu(s, pairs_per_collider=4)
    g.step(); g.synchronize()
    o.step()
    assert pair_set(g.pairs()[:, 1:]) == pair_set(o.pairs())
    assert tight.counts()["error"] == 0 and g.counts()["error"] == 0
