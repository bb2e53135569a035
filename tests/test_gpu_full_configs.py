"""GPU parity at the full sizes of the benchmark workloads.

The same checks as tests/test_gpu_parity.py, on the workloads the benchmark runs:
  * the 20-row box pyramid (210 cubes), all 600 frames of its run;
  * 65,536 mixed bodies over a 256 x 256-cell heightfield (131,072 triangles);
  * 2048 capsule chains of 32 links (65,536 bodies, 65,536 joints);
  * all 4096 scenes of the batched workload as one world (1.69 M simulated bodies),
    launched from a CUDA graph as the benchmark's frame is.

Each run checks, against the CPU oracle:
  * creation bounds, bit for bit;
  * broadphase pair sets on frames 1 and 10 (and later pyramid frames), as sets;
  * manifold normals, points and target velocities on those frames, within 1e-5;
  * every frame's body state within 1e-5 relative, with the oracle fed the GPU's
    colour-sorted contact order (frames run in lockstep, so the poses that the
    manifold checks start from are the same on both sides).
"""
import numpy as np
import pytest

from physecs_gb300 import scenes
from tests.parity import compare_contacts, gpu_keys, pair_set, rel_state_diff

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _check_creation_bounds(g, o, s):
    gb = g.bounds()
    ids, ob = o.bounds()
    order = np.array([s.arrays["collider_start"][e] + c for e, c in ids])
    assert np.array_equal(gb[order].view(np.uint32), ob.view(np.uint32))


def _lockstep_single(s, frames, check, **kw):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    g = World([s], **kw)
    o = OracleScene(s)
    _check_creation_bounds(g, o, s)
    seen = {}
    for f in range(1, frames + 1):
        g.step()
        g.synchronize()
        ids, gf, meta = g.contacts()
        keys = gpu_keys(ids, meta)
        o.set_contact_order(keys)
        o.step()
        assert o.order_error() == 0, "frame %d: GPU manifolds not found in the oracle" % f
        if f in check:
            gp, op = pair_set(g.pairs()[:, 1:]), pair_set(o.pairs())
            assert gp == op, "frame %d: %d GPU pairs, %d oracle pairs, %d common" % (f, len(gp), len(op), len(gp & op))
            _, of = o.contacts()
            worst = compare_contacts(keys, gf, o.contact_keys(), of)
            assert worst <= TOL, "frame %d: manifolds differ by %g" % (f, worst)
            seen[f] = (len(gp), len(keys))
        d = rel_state_diff(g.read_bodies(), o.state())
        assert d <= TOL, "frame %d: relative state difference %g" % (f, d)
    assert g.counts()["error"] == 0
    g.close()
    o.close()
    return seen


def test_pyramid_20_rows_all_600_frames(gpu_lib, oracle_lib):
    """The 210-cube pyramid at dt 1/60, 4 substeps, 8 iterations, for the whole run."""
    seen = _lockstep_single(scenes.pyramid(), 600, (1, 10, 100, 300, 600))
    assert seen[1][0] == 20 and seen[600][1] > 0


def test_large_mixed_65536_bodies_on_a_heightfield(gpu_lib, oracle_lib):
    """65,536 mixed bodies (boxes, spheres, capsules, hulls) over 131,072 triangles."""
    s = scenes.large_mixed()
    assert s.n_dynamic == 65536 and len(s.arrays["tri_indices"]) == 3 * 131072
    seen = _lockstep_single(s, 10, (1, 10))
    assert seen[10][0] > 65536 and seen[10][1] > 0


def test_joint_chains_2048_by_32(gpu_lib, oracle_lib):
    """2048 chains of 32 capsule links under one static ceiling (65,536 joints, most of
    the root joints in the serially solved overflow colour), 8 substeps, 4 iterations."""
    s = scenes.joint_chains()
    assert s.n_dynamic == 65536 and len(s.arrays["joint_type"]) == 65536
    _lockstep_single(s, 10, (1, 10))


def _per_scene(rows, scene_col, n):
    """Split rows by their scene column (stable, so each scene keeps the GPU's order)."""
    order = np.argsort(rows[:, scene_col], kind="stable")
    cut = np.searchsorted(rows[order, scene_col], np.arange(n + 1))
    return order, cut


def test_batched_4096_scenes_as_one_graph_launched_world(gpu_lib, oracle_lib):
    """All 4096 scenes of the batched workload in one world replaying its CUDA graph:
    every scene equals its own oracle run, checked in parallel worker processes."""
    from physecs_gb300.api import World
    from tests.oracle_pool import OraclePool, _build_scene
    n = 4096
    specs = [("batch", i, 4) for i in range(n)]
    ss = [_build_scene(sp) for sp in specs]
    pool = OraclePool(specs, [len(s.arrays["pos"]) for s in ss])
    try:
        g = World(ss, use_graph=True)
        bs = g.body_start
        cs = np.cumsum([0] + [len(s.arrays["col_type"]) for s in ss])
        gb = g.bounds()
        r = pool.check_bounds([gb[cs[i]:cs[i + 1]] for i in range(n)])
        assert r["bounds_mismatch"] == [], r["bounds_mismatch"][:10]
        for f in range(1, 11):
            g.step()
            g.synchronize()
            ids, gf, meta = g.contacts()
            order, cut = _per_scene(ids, 0, n)
            keys = gpu_keys(ids[order], meta[order])
            gf = gf[order]
            st = g.read_bodies()
            states = [{k: v[bs[i]:bs[i + 1]] for k, v in st.items()} for i in range(n)]
            kl = [keys[cut[i]:cut[i + 1]] for i in range(n)]
            pairs = contacts = None
            if f in (1, 10):
                gp = g.pairs()
                po, pc = _per_scene(gp, 0, n)
                gp = gp[po]
                pairs = [gp[pc[i]:pc[i + 1], 1:] for i in range(n)]
                contacts = [(kl[i], gf[cut[i]:cut[i + 1]]) for i in range(n)]
            r = pool.step(kl, states, pairs, contacts)
            assert r["order_error"] == 0, "frame %d: GPU manifolds not found in the oracle" % f
            assert r["pair_mismatch"] == [], "frame %d: pair sets differ in scenes %s" % (f, r["pair_mismatch"][:10])
            assert r["manifolds"] <= TOL, "frame %d: manifolds differ by %g" % (f, r["manifolds"])
            assert r["state"] <= TOL, "frame %d: relative state difference %g" % (f, r["state"])
        c = g.counts()
        assert c["error"] == 0 and c["scenes"] == n and c["simulated"] > 1_600_000
        g.close()
    finally:
        pool.close()
