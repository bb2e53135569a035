"""The CPU oracle against golden vectors produced by the unmodified reference.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py, which
runs Physecs' own Scene::simulate / physecs::collision (compiled from its
sources).  Every comparison is bit-exact: the oracle repeats the reference's
float operation order.
"""
import os

import numpy as np
import pytest

from physecs_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def _golden_scenes():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MG = _golden_scenes()
SCENES = MG.golden_scenes()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_scene_generator_stable(name):
    """The seeded scene generator still produces the scenes the fixtures were made from."""
    g = _load("frames_%s.npz" % name)
    assert str(g["scene_sha256"]) == MG.scene_hash(SCENES[name][0])


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_matches_reference_frames(oracle_lib, name):
    g = _load("frames_%s.npz" % name)
    s, frames = SCENES[name]
    o = oracle_lib.OracleScene(s)
    ids, b = o.bounds()
    np.testing.assert_array_equal(ids, g["bounds_ids"])
    np.testing.assert_array_equal(b, g["bounds"])
    f = 0
    for target in frames:
        while f < target:
            o.step()
            f += 1
            if f == 1:
                np.testing.assert_array_equal(o.pairs(), g["pairs_f1"])
                cid, cf = o.contacts()
                np.testing.assert_array_equal(cid, g["contacts_f1_ids"])
                np.testing.assert_array_equal(cf, g["contacts_f1"])
        st = o.state()
        for k, v in st.items():
            np.testing.assert_array_equal(v, g["state_f%d_%s" % (f, k)], err_msg="%s frame %d %s" % (name, f, k))


def _kat_cases():
    g = _load("narrow_pairs.npz")
    return sorted({k.rsplit("__", 1)[0] for k in g})


SHAPES = {
    "sphere": (scenes.SPHERE, [0.5]),
    "capsule": (scenes.CAPSULE, [0.4, 0.3]),
    "box": (scenes.BOX, [0.5, 0.4, 0.3]),
    "hull": (scenes.CONVEX_MESH, [0.8, 0.8, 0.8]),
    "boxhull": (scenes.CONVEX_MESH, [1.0, 1.0, 1.0]),
}


def _meshes():
    hull = scenes.convex_hull(np.asarray(scenes._hull_pool(scenes.SplitMix64(7), count=1)[0][0]))
    box_hull = scenes.box_hull((0.5, 0.4, 0.3))
    tri = scenes.heightfield(scenes.SplitMix64(5), cells=6, amplitude=0.3, lattice=3)
    return {"hull": hull, "boxhull": box_hull, "trimesh": (tri[0], tri[1])}


@pytest.mark.parametrize("case", _kat_cases())
def test_oracle_narrowphase_kat(oracle_lib, case):
    """physecs::collision known answers for every shape pair (touching poses)."""
    g = _load("narrow_pairs.npz")
    poses = g[case + "__poses"]
    ids_ref, f_ref = g[case + "__ids"], g[case + "__f"]
    a, b = case.split("__")
    meshes = _meshes()
    ta, pa = SHAPES[a]
    rows_ids, rows_f = [], []
    for i, p in enumerate(poses):
        if b == "trimesh":
            s = scenes.pair_scene(ta, pa, (p[0:3], p[3:7]), scenes.TRIANGLE_MESH, [], ([0, 0, 0], scenes.IDENTITY_Q),
                                  mesh0=meshes.get(a), mesh1=meshes["trimesh"], dynamic=(True, False))
        else:
            tb, pb = SHAPES[b]
            s = scenes.pair_scene(ta, pa, (p[0:3], p[3:7]), tb, pb, (p[7:10], p[10:14]),
                                  mesh0=meshes.get(a), mesh1=meshes.get(b))
        ids, f = oracle_lib.OracleScene(s).collide([[0, 0, 1, 0]])
        for k in range(len(ids)):
            rows_ids.append([i] + list(ids[k][1:3]))
            rows_f.append(f[k])
    rows_ids = np.asarray(rows_ids, np.int32).reshape(-1, 3)
    rows_f = np.asarray(rows_f, np.float32).reshape(-1, 28)
    np.testing.assert_array_equal(rows_ids, ids_ref)
    np.testing.assert_array_equal(rows_f, f_ref)


def test_kat_covers_every_shape_pair():
    cases = set(_kat_cases())
    for a in SHAPES:
        assert "%s__trimesh" % a in cases
        for b in SHAPES:
            assert "%s__%s" % (a, b) in cases
    g = _load("narrow_pairs.npz")
    # the poses produce real contacts, not only separations
    assert sum(len(g[c + "__ids"]) for c in cases) > 200


def _ref_available():
    try:
        from oracle.ref import ref_api
        return ref_api.available()
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="oracle/_ref (the reference built from its sources) is not built here")
def test_oracle_matches_live_reference_on_flagged_scenes(oracle_lib):
    """Kinematic bodies, triggers, disabled colliders, no dynamic bodies, no contacts."""
    from oracle.ref.ref_api import RefScene
    from tests.scene_variants import apart_scene, flagged_scene, static_only_scene
    for s in (flagged_scene(), static_only_scene(), apart_scene(), flagged_scene(32, 40)):
        o, r = oracle_lib.OracleScene(s), RefScene(s)
        for f in range(30):
            o.step()
            r.step()
            a, b = o.state(), r.state()
            for k in a:
                np.testing.assert_array_equal(a[k], b[k], err_msg="frame %d %s" % (f, k))
        np.testing.assert_array_equal(o.pairs(), r.pairs())


@pytest.mark.skipif(not _ref_available(), reason="oracle/_ref (the reference built from its sources) is not built here")
@pytest.mark.parametrize("seed,n,chain", [(11, 300, 0.0), (12, 200, 1.0), (13, 1500, 0.3)])
def test_oracle_matches_live_reference(oracle_lib, seed, n, chain):
    """Where the reference library is built, run both side by side for 40 frames."""
    from oracle.ref.ref_api import RefScene
    s = scenes.batch_scene(seed, n_bodies=n, chain_prob=chain)
    o, r = oracle_lib.OracleScene(s), RefScene(s)
    for f in range(40):
        o.step()
        r.step()
        a, b = o.state(), r.state()
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg="frame %d %s" % (f, k))


def test_oracle_contact_order_keys_round_trip(oracle_lib):
    """The ordering hook the GPU lockstep tests use: a frame's contact keys (entity,
    collider within the body, triangle) fed to a second oracle at the same state all
    match, in any order; a key that names no contact is counted, and so is the contact
    it leaves without a key."""
    from oracle.port_api import OracleScene
    s = scenes.batch_scene(8, n_bodies=80, chain_prob=1.0)
    a = OracleScene(s)
    for _ in range(3):
        a.step()
    keys = a.contact_keys()
    assert len(keys) > 20
    for order in (keys, keys[::-1]):
        b = OracleScene(s)
        for _ in range(2):
            b.step()
        b.set_contact_order(order)
        b.step()
        assert b.order_error() == 0
    bad = keys.copy()
    bad[0, 1] += 100
    c = OracleScene(s)
    for _ in range(2):
        c.step()
    c.set_contact_order(bad)
    c.step()
    assert c.order_error() == 2
