#!/usr/bin/env python3
"""Generate golden fixtures from the UNMODIFIED Physecs reference (oracle/_ref).

Physecs ships no tests and no golden vectors, so every fixture here is produced
by running the reference itself (built from its own sources by
oracle/ref/build_ref.py) on seeded scenes from physecs_gb300.scenes:

  frames_<name>.npz    creation bounds, first-frame pair set and contact rows,
                       and body state after selected frames, for whole scenes
  narrow_pairs.npz     manifolds of physecs::collision for every shape pair at
                       seeded touching poses (known-answer tests)
  queries.npz          Scene::raycastClosest and Scene::overlap answers on stepped
                       scenes for seeded rays and shapes
  triggers.npz         the onTriggerEnter / onTriggerExit callbacks of stepped scenes
                       with trigger colliders
  trimesh_bvh.npz      physecs::TriangleMesh's triangles and BVH nodes for seeded meshes,
                       degenerate ones included
  deltas.npz           body states of scenes stepped with seeded registry deltas (patched
                       poses, written velocities, setIsKinematic) between frames
  filters.npz          body states and trigger events of a scene stepped under a user
                       contact filter, with setCanCollide toggled between frames
  topology.npz         entity values and body states of a scene whose entities are
                       destroyed and created between frames
  mechanisms.npz       body states of every joint kind with drives, limits, a servo and
                       a gear, with joint setters and registry edits between frames

Run in a checkout with the reference present:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from physecs_gb300 import scenes  # noqa: E402


def scene_hash(s):
    h = hashlib.sha256()
    for k in sorted(s.arrays):
        h.update(k.encode())
        h.update(np.ascontiguousarray(s.arrays[k]).tobytes())
    return h.hexdigest()


def golden_scenes():
    """name -> (scene, frames at which state is recorded)."""
    return {
        "pyramid": (scenes.pyramid(), [1, 2, 5, 10, 30, 60]),
        "mixed_a": (scenes.batch_scene(101, n_bodies=60), [1, 5, 20]),
        "mixed_b": (scenes.batch_scene(202, n_bodies=120), [1, 5, 20]),
        "chain": (scenes.batch_scene(303, n_bodies=30, chain_prob=1.0), [1, 5, 20]),
        "joints": (scenes.joint_chains(n_chains=12, links=6), [1, 5, 20, 40]),
        "heightfield": (scenes.large_mixed(n_bodies=300, cells=32), [1, 3, 6]),
    }


def pair_poses(rng, n):
    """Seeded poses that put two unit-ish shapes within touching distance."""
    p0 = np.zeros((n, 3))
    d = rng.normal(3 * n).reshape(n, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p1 = d * rng.uniform(n, 0.3, 1.6)[:, None]
    return p0, rng.quaternions(n), p1, rng.quaternions(n)


def narrow_kat():
    from oracle.ref.ref_api import RefScene
    rng = scenes.SplitMix64(0x5EED0000 + 99)
    hull = scenes.convex_hull(np.asarray(scenes._hull_pool(scenes.SplitMix64(7), count=1)[0][0]))
    box_hull = scenes.box_hull((0.5, 0.4, 0.3))
    shapes = {
        "sphere": (scenes.SPHERE, [0.5], None),
        "capsule": (scenes.CAPSULE, [0.4, 0.3], None),
        "box": (scenes.BOX, [0.5, 0.4, 0.3], None),
        "hull": (scenes.CONVEX_MESH, [0.8, 0.8, 0.8], hull),
        "boxhull": (scenes.CONVEX_MESH, [1.0, 1.0, 1.0], box_hull),
    }
    out = {}
    n = 40
    for a, (ta, pa, ma) in shapes.items():
        for b, (tb, pb, mb) in shapes.items():
            p0, q0, p1, q1 = pair_poses(rng, n)
            rows_ids, rows_f = [], []
            for i in range(n):
                s = scenes.pair_scene(ta, pa, (p0[i], q0[i]), tb, pb, (p1[i], q1[i]), mesh0=ma, mesh1=mb)
                r = RefScene(s)
                ids, f = r.collide([[0, 0, 1, 0]])
                for k in range(len(ids)):
                    rows_ids.append([i] + list(ids[k][1:3]))
                    rows_f.append(f[k])
            key = "%s__%s" % (a, b)
            out[key + "__poses"] = np.concatenate([p0, q0, p1, q1], axis=1).astype(np.float32)
            out[key + "__ids"] = np.asarray(rows_ids, np.int32).reshape(-1, 3)
            out[key + "__f"] = np.asarray(rows_f, np.float32).reshape(-1, 28)
    # shapes against a small triangle mesh (a 6x6 heightfield patch)
    tri = scenes.heightfield(scenes.SplitMix64(5), cells=6, amplitude=0.3, lattice=3)
    for a, (ta, pa, ma) in shapes.items():
        p0 = np.stack([rng.uniform(n, -2, 2), 0.2 + rng.uniform(n, 0, 0.6), rng.uniform(n, -2, 2)], axis=1)
        q0 = rng.quaternions(n)
        rows_ids, rows_f = [], []
        for i in range(n):
            s = scenes.pair_scene(ta, pa, (p0[i], q0[i]), scenes.TRIANGLE_MESH, [], ([0, 0, 0], scenes.IDENTITY_Q),
                                  mesh0=ma, mesh1=(tri[0], tri[1]), dynamic=(True, False))
            r = RefScene(s)
            ids, f = r.collide([[0, 0, 1, 0]])
            for k in range(len(ids)):
                rows_ids.append([i] + list(ids[k][1:3]))
                rows_f.append(f[k])
        key = "%s__trimesh" % a
        out[key + "__poses"] = np.concatenate([p0, q0, np.zeros((n, 3)), np.tile([0, 0, 0, 1.0], (n, 1))], axis=1).astype(np.float32)
        out[key + "__ids"] = np.asarray(rows_ids, np.int32).reshape(-1, 3)
        out[key + "__f"] = np.asarray(rows_f, np.float32).reshape(-1, 28)
    return out


def query_scenes():
    """name -> (scene, frames stepped before the queries)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import flagged_scene
    return {
        "mixed": (scenes.batch_scene(12, n_bodies=200), 30),
        "flagged": (flagged_scene(), 10),
        "heightfield": (scenes.large_mixed(n_bodies=300, cells=32), 5),
    }


def query_inputs(s, pos, seed):
    """Seeded rays (8 floats: unused, origin, dir, max distance) aimed at bodies, a
    quarter of them exactly vertical and some starting inside a body; a per-body accept
    table; and overlap shapes of every kind around bodies."""
    rng = scenes.SplitMix64(0x5EED0000 + seed)
    nb = len(pos)
    n = 256
    tgt = pos[(rng.uniform(n) * nb).astype(int) % nb] + 0.6 * rng.normal(3 * n).reshape(n, 3)
    org = tgt + np.array([0.0, 15.0, 0.0]) + 2.0 * rng.normal(3 * n).reshape(n, 3)
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    vert = np.arange(n) % 4 == 0
    org[vert] = tgt[vert] + np.array([0.0, 15.0, 0.0])
    d[vert] = np.array([0.0, -1.0, 0.0])
    inside = np.arange(n) % 16 == 1
    org[inside] = pos[(np.arange(n)[inside] * 7) % nb]
    rays = np.zeros((n, 8), np.float32)
    rays[:, 1:4], rays[:, 4:7] = org, d
    rays[:, 7] = rng.uniform(n, 4.0, 40.0)
    accept = (rng.uniform(nb) < 0.8).astype(np.uint8)
    m = 96
    kinds = (np.arange(m) % 4).astype(np.int32)
    if not s.convex:
        kinds[kinds == 3] = 2
    qpos = pos[(rng.uniform(m) * nb).astype(int) % nb] + 0.7 * rng.normal(3 * m).reshape(m, 3)
    qquat = rng.quaternions(m)
    prm = np.zeros((m, 3), np.float32)
    u = rng.uniform(3 * m).reshape(m, 3)
    prm[kinds == 0, 0] = 0.2 + 1.3 * u[kinds == 0, 0]
    prm[kinds == 1, 0] = 0.2 + 0.8 * u[kinds == 1, 0]
    prm[kinds == 1, 1] = 0.1 + 0.5 * u[kinds == 1, 1]
    prm[kinds == 2] = 0.2 + 1.0 * u[kinds == 2]
    prm[kinds == 3] = 0.5 + u[kinds == 3]
    mesh = np.where(kinds == 3, 0, -1).astype(np.int32)
    filt = np.where(np.arange(m) % 3 == 2, 1, 0).astype(np.int32)
    return rays, accept, qpos.astype(np.float32), qquat.astype(np.float32), kinds, prm, mesh, filt


def mtd_sorted(hits):
    """overlapWithMinTranslationalDistance records in a canonical order (the reference
    lists them in its tree's order): by body, collider, then the float bits."""
    return sorted(hits, key=lambda h: (h[0], h[1], tuple(np.asarray(list(h[2]) + [h[3]], np.float32).view(np.uint32))))


def query_fixture():
    from oracle.ref.ref_api import RefScene
    out = {}
    for si, (name, (s, frames)) in enumerate(query_scenes().items()):
        r = RefScene(s)
        for _ in range(frames):
            r.step()
        rays, accept, qpos, qquat, kinds, prm, mesh, filt = query_inputs(s, r.state()["pos"], 500 + si)
        hit = r.raycast(rays, accept)
        nohit = r.raycast(rays, None)
        starts, flat = [0], []
        for k in range(len(kinds)):
            hs = sorted(r.overlap(qpos[k], qquat[k], kinds[k], prm[k], mesh[k], filt[k]))
            flat.extend(hs)
            starts.append(len(flat))
        mstarts, mids, mf = [0], [], []
        for k in range(len(kinds)):
            for b, c, nrm, mtd in mtd_sorted(r.overlap_mtd(qpos[k], qquat[k], kinds[k], prm[k], mesh[k])):
                mids.append((b, c))
                mf.append(list(nrm) + [mtd])
            mstarts.append(len(mids))
        pre = name + "__"
        out.update({pre + "scene_sha256": np.array(scene_hash(s)), pre + "frames": np.array(frames, np.int32),
                    pre + "rays": rays, pre + "accept": accept, pre + "ray_body": hit["body"], pre + "ray_pos": hit["pos"],
                    pre + "ray_body_nofilter": nohit["body"], pre + "q_pos": qpos, pre + "q_quat": qquat,
                    pre + "q_type": kinds, pre + "q_params": prm, pre + "q_mesh": mesh, pre + "q_filter": filt,
                    pre + "q_start": np.asarray(starts, np.int32), pre + "q_hits": np.asarray(flat, np.int32).reshape(-1, 2),
                    pre + "mtd_start": np.asarray(mstarts, np.int32), pre + "mtd_ids": np.asarray(mids, np.int32).reshape(-1, 2),
                    pre + "mtd_f": np.asarray(mf, np.float32).reshape(-1, 4)})
    return out


def trimesh_cases():
    """name -> (vertices (n, 3) float32, indices (3t,) uint32): meshes for the BVH build,
    with the cases that steer its branches: axes without extent, triangles that share a
    centroid (no split separates them), zero-area and duplicate triangles, signed zeros,
    a skewed distribution, a single triangle and an empty mesh."""
    rng = np.random.default_rng(0x7215)
    out = {}
    v, ix, _ = scenes.heightfield(scenes.SplitMix64(scenes.scene_seed(2, 77)), cells=12, lattice=4)
    out["heightfield12"] = (v, ix.ravel())
    n = 300
    v = rng.uniform(-5, 5, (3 * n, 3)).astype(np.float32)
    v[rng.random(3 * n) < 0.1, 1] = np.float32(-0.0)
    v[rng.random(3 * n) < 0.1, 0] = np.float32(0.0)
    ix = np.arange(3 * n, dtype=np.uint32)
    dup = rng.integers(0, n, 40)
    ix = np.concatenate([ix, ix.reshape(-1, 3)[dup].ravel()])
    deg = rng.integers(0, 3 * n, 20)
    ix = np.concatenate([ix, np.repeat(deg, 3).astype(np.uint32)])          # zero-area triangles
    out["soup"] = (v, ix.astype(np.uint32))
    xs = np.arange(11, dtype=np.float32)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    v = np.stack([X.ravel(), np.zeros(121, np.float32), Z.ravel()], axis=1).astype(np.float32)
    q = np.arange(10)
    I, J = np.meshgrid(q, q, indexing="ij")
    a, b, c, d = (I * 11 + J).ravel(), ((I + 1) * 11 + J).ravel(), (I * 11 + J + 1).ravel(), ((I + 1) * 11 + J + 1).ravel()
    out["flat"] = (v, np.stack([a, c, b, b, c, d], axis=1).ravel().astype(np.uint32))
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    out["single"] = (v, np.array([0, 1, 2], np.uint32))
    out["same_centroid"] = (v, np.tile(np.array([0, 1, 2], np.uint32), 90))
    k = np.arange(400)
    x = (1.3 ** (k / 10.0)).astype(np.float32)      # exponentially spaced: lopsided splits
    z0 = np.zeros_like(x)
    v = np.stack([np.stack([x, z0, z0], 1), np.stack([x + 0.5, z0 + 1, z0], 1), np.stack([x, z0, z0 + 1], 1)], 1)
    v = v.reshape(-1, 3).astype(np.float32)
    out["skewed"] = (v, (rng.permutation(400).repeat(3) * 3 + np.tile(np.arange(3), 400)).astype(np.uint32))
    out["empty"] = (v[:3], np.zeros(0, np.uint32))
    return out


def trimesh_fixture():
    from oracle.ref.ref_api import trimesh_build
    out = {}
    for name, (v, ix) in trimesh_cases().items():
        if not len(ix):
            continue   # the reference's constructor throws for a mesh without triangles
        tris, nodes = trimesh_build(v, ix)
        out.update({name + "__verts": v, name + "__indices": ix, name + "__tris": tris, name + "__nodes": nodes})
    return out


def delta_scenes():
    """name -> (scene, frames stepped, frames whose state is recorded)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import flagged_scene
    return {
        "flagged": (flagged_scene(), 40, [10, 20, 40]),
        "chains": (scenes.joint_chains(n_chains=4, links=6), 40, [10, 20, 40]),
    }


def delta_fixture():
    from oracle.ref.ref_api import RefScene
    from physecs_gb300.api import pack_deltas
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import delta_schedule
    out = {}
    for name, (s, frames, rec) in delta_scenes().items():
        sch = delta_schedule(s, frames)
        r = RefScene(s)
        pre = name + "__"
        out[pre + "scene_sha256"] = np.array(scene_hash(s))
        for f in range(frames):
            if f in sch:
                r.apply_deltas(pack_deltas(sch[f]))
            r.step()
            if f + 1 in rec:
                for k, v in r.state().items():
                    out[pre + "f%d_%s" % (f + 1, k)] = v
    return out


def filter_case():
    """(scene, filter, can-collide schedule {frame: (body0, body1, can)}, frames, recorded
    frames): colliders get data values 0..3; pairs with a trigger, or whose data share
    bit 1, are trigger pairs."""
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import flagged_scene
    s = flagged_scene(seed=8, n=90)
    a = s.arrays
    a["col_data"][:] = np.random.default_rng(4).integers(0, 4, len(a["col_data"]))

    def filt(t0, d0, t1, d1):
        return 1 if (t0 or t1 or (d0 & d1 & 2)) else 0
    return s, filt, {10: (5, 6, False), 30: (5, 6, True), 35: (7, 12, False)}, 50, [20, 50]


def filter_fixture():
    from oracle.ref.ref_api import RefScene
    s, filt, cc, frames, rec = filter_case()
    r = RefScene(s)
    r.set_contact_filter(filt)
    out = {"scene_sha256": np.array(scene_hash(s))}
    for f in range(frames):
        if f in cc:
            r.set_can_collide(*cc[f])
        r.step()
        if f + 1 in rec:
            for k, v in r.state().items():
                out["f%d_%s" % (f + 1, k)] = v
    out["events"] = events_sorted(r.trigger_events())
    return out


def topology_case():
    """(scene, schedule, frames, recorded frames) for entities destroyed and created
    between frames (tests/scene_variants.py topology_schedule)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import topology_schedule
    s = scenes.batch_scene(11, n_bodies=60, chain_prob=0.0)
    return s, topology_schedule(s, 60, seed=11), 60, [30, 60]


def joint_topology_case():
    """(scene, plan {frame: ("destroy", joint) | ("create", (type, body0, body1))}, anchor
    frames, frames): capsule chains whose joints are destroyed and created between frames,
    a joint made between frames destroyed again among them."""
    s = scenes.joint_chains(n_chains=4, links=6)
    nj = len(s.arrays["joint_type"])
    fr = np.zeros(14, np.float32)
    fr[1], fr[6], fr[8], fr[13] = -0.35, 1.0, 0.35, 1.0
    plan = {8: ("destroy", 3), 12: ("create", (scenes.JOINT_SPHERICAL, 6, 12)), 20: ("destroy", 10),
            25: ("create", (scenes.JOINT_REVOLUTE, 18, 24)), 30: ("destroy", nj), 35: ("create", (scenes.JOINT_FIXED, 2, 9))}
    return s, plan, fr, 50


def _collider_scene(typ, prm, pos=(0.0, 0.0, 0.0)):
    s = scenes.SceneData("collider")
    s.add_bodies(pos=[[0.0, 0.0, 0.0]], quat=[scenes.IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3),
                 inv_inertia=np.zeros(9), col_type=typ, col_params=prm, col_pos=list(pos))
    return s.finalize()


def collider_topology_case():
    """(scene, plan {frame: [("clear", body) | ("add", body, collider SceneData)]}, frames):
    colliders cleared from and added to dynamic and static bodies between frames."""
    s = scenes.batch_scene(14, n_bodies=50, chain_prob=0.0)
    dyn = [int(b) for b in np.nonzero(s.arrays["flags"] & scenes.BODY_DYNAMIC)[0]]
    plan = {5: [("clear", dyn[0])],
            9: [("add", dyn[1], _collider_scene(scenes.SPHERE, [0.3, 0, 0, 0], (0.4, 0, 0)))],
            14: [("add", dyn[0], _collider_scene(scenes.BOX, [0.3, 0.3, 0.3, 0]))],
            20: [("add", 0, _collider_scene(scenes.BOX, [1.0, 0.2, 1.0, 0], (0, 1.0, 0))), ("clear", dyn[2])],
            26: [("add", dyn[2], _collider_scene(scenes.CAPSULE, [0.3, 0.2, 0, 0])),
                 ("add", dyn[2], _collider_scene(scenes.SPHERE, [0.2, 0, 0, 0], (0, 0.5, 0)))]}
    return s, plan, 50


def run_collider_plan(sim, plan, frames):
    for f in range(frames):
        for act in plan.get(f, []):
            if act[0] == "clear":
                sim.clear_colliders(act[1])
            else:
                sim.add_collider(act[1], act[2])
        sim.step()
    return sim.state()


def run_joint_plan(sim, plan, fr, frames):
    for f in range(frames):
        if f in plan:
            kind, arg = plan[f]
            if kind == "destroy":
                sim.destroy_joint(arg)
            else:
                sim.create_joint(arg[0], arg[1], arg[2], fr)
        sim.step()
    return sim.state()


def topology_fixture():
    from oracle.ref.ref_api import RefScene
    s, sch, frames, rec = topology_case()
    r = RefScene(s)
    out = {"scene_sha256": np.array(scene_hash(s))}
    js, plan, fr, jframes = joint_topology_case()
    out["joints_scene_sha256"] = np.array(scene_hash(js))
    for k, v in run_joint_plan(RefScene(js), plan, fr, jframes).items():
        out["joints_f%d_%s" % (jframes, k)] = v
    cs, cplan, cframes = collider_topology_case()
    out["colliders_scene_sha256"] = np.array(scene_hash(cs))
    for k, v in run_collider_plan(RefScene(cs), cplan, cframes).items():
        out["colliders_f%d_%s" % (cframes, k)] = v
    ents = []
    for f in range(frames):
        if f in sch:
            kill, spawn = sch[f]
            for b in kill:
                r.destroy_body(b)
            for sp in spawn:
                ents.append(r.create_body(sp)[1])
        r.step()
        if f + 1 in rec:
            for k, v in r.state().items():
                out["f%d_%s" % (f + 1, k)] = v
    out["entities"] = np.asarray(ents, np.uint32)
    return out


def trigger_scenes():
    """name -> (scene, frames stepped)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import flagged_scene, trigger_scene
    return {
        "zones_a": (trigger_scene(41), 120),
        "zones_b": (trigger_scene(42), 120),
        "flagged": (flagged_scene(), 60),
    }


def events_sorted(ev):
    """Trigger events (frame, kind, body0, collider0, body1, collider1) in a canonical
    order: the reference calls them in its hash set's order within a frame."""
    ev = np.asarray(ev, np.int32).reshape(-1, 6)
    return ev[np.lexsort(ev.T[::-1])] if len(ev) else ev


def trigger_fixture():
    from oracle.ref.ref_api import RefScene
    out = {}
    for name, (s, frames) in trigger_scenes().items():
        r = RefScene(s)
        for _ in range(frames):
            r.step()
        pre = name + "__"
        out.update({pre + "scene_sha256": np.array(scene_hash(s)), pre + "frames": np.array(frames, np.int32),
                    pre + "events": events_sorted(r.trigger_events())})
    return out


MECHANISM_FRAMES, MECHANISM_RECORDED = 120, [10, 30, 60, 120]


def mechanism_fixture():
    from oracle.ref.ref_api import RefScene
    sys.path.insert(0, os.path.dirname(HERE))
    from scene_variants import apply_mechanism_op, mechanism_ops, mechanism_scene
    s, info = mechanism_scene()
    ops = mechanism_ops(s, info)
    r = RefScene(s)
    out = {"scene_sha256": np.array(scene_hash(s))}
    for f in range(MECHANISM_FRAMES):
        for op in ops:
            if op[0] == f:
                apply_mechanism_op(r, op)
        r.step()
        if f + 1 in MECHANISM_RECORDED:
            for k, v in r.state().items():
                out["f%d_%s" % (f + 1, k)] = v
    return out


def main():
    from oracle.ref import build_ref, ref_api
    if not ref_api.available():
        build_ref.build()
    from oracle.ref.ref_api import RefScene
    for name, (s, frames) in golden_scenes().items():
        r = RefScene(s)
        ids, b = r.bounds()
        rec = {"scene_sha256": np.array(scene_hash(s)), "bounds_ids": ids, "bounds": b}
        f = 0
        for target in frames:
            while f < target:
                r.step()
                f += 1
                if f == 1:
                    rec["pairs_f1"] = r.pairs()
                    cid, cf = r.contacts()
                    rec["contacts_f1_ids"], rec["contacts_f1"] = cid, cf
            st = r.state()
            for k, v in st.items():
                rec["state_f%d_%s" % (f, k)] = v
        rec["frames"] = np.array(frames, np.int32)
        np.savez_compressed(os.path.join(HERE, "frames_%s.npz" % name), **rec)
        print(name, "ok")
    np.savez_compressed(os.path.join(HERE, "narrow_pairs.npz"), **narrow_kat())
    print("narrow_pairs ok")
    np.savez_compressed(os.path.join(HERE, "queries.npz"), **query_fixture())
    print("queries ok")
    np.savez_compressed(os.path.join(HERE, "triggers.npz"), **trigger_fixture())
    print("triggers ok")
    np.savez_compressed(os.path.join(HERE, "trimesh_bvh.npz"), **trimesh_fixture())
    print("trimesh_bvh ok")
    np.savez_compressed(os.path.join(HERE, "deltas.npz"), **delta_fixture())
    print("deltas ok")
    np.savez_compressed(os.path.join(HERE, "filters.npz"), **filter_fixture())
    print("filters ok")
    np.savez_compressed(os.path.join(HERE, "topology.npz"), **topology_fixture())
    print("topology ok")
    np.savez_compressed(os.path.join(HERE, "mechanisms.npz"), **mechanism_fixture())
    print("mechanisms ok")


if __name__ == "__main__":
    main()
