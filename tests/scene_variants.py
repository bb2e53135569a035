"""Scenes that exercise the reference's less common inputs: kinematic bodies (moving,
never integrated), trigger colliders (no contacts), colliders with enableSimulation
off (no pairs), a scene without dynamic bodies and a scene without any contact."""
import numpy as np

from physecs_gb300 import scenes
from physecs_gb300.scenes import character_moves, character_scene, strip_colliders  # noqa: F401


def flagged_scene(seed=31, n=80):
    s = scenes.batch_scene(seed, n_bodies=n)
    a = s.arrays
    rng = np.random.default_rng(seed)
    dyn = np.nonzero(a["flags"] & scenes.BODY_DYNAMIC)[0]
    kin = rng.choice(dyn, size=max(1, len(dyn) // 10), replace=False)
    a["flags"][kin] |= scenes.BODY_KINEMATIC
    a["vel"][kin] = rng.normal(size=(len(kin), 3)).astype(np.float32)
    a["ang_vel"][kin] = rng.normal(size=(len(kin), 3)).astype(np.float32)
    ncol = len(a["col_type"])
    cols = rng.permutation(np.arange(1, ncol))          # collider 0 is the ground
    a["col_is_trigger"][cols[: ncol // 10]] = 1
    a["col_enable_sim"][cols[ncol // 10: ncol // 5]] = 0
    return s


def static_only_scene():
    """Two static boxes overlapping: no dynamic body, so no pair at all."""
    s = scenes.pair_scene(scenes.BOX, [0.5, 0.5, 0.5], ([0, 0, 0], scenes.IDENTITY_Q), scenes.BOX, [0.5, 0.5, 0.5],
                          ([0.3, 0, 0], scenes.IDENTITY_Q), dynamic=(False, False))
    return s


def apart_scene():
    """Two dynamic spheres far apart: pairs but no manifold."""
    return scenes.pair_scene(scenes.SPHERE, [0.5], ([0, 5, 0], scenes.IDENTITY_Q), scenes.SPHERE, [0.5],
                             ([10, 5, 0], scenes.IDENTITY_Q))


def trigger_scene(seed=41, n=90):
    """Trigger volumes in the path of falling bodies: four static trigger colliders (a
    box slab, a sphere, a capsule and a convex hull) above a ground box, mixed dynamic
    bodies dropped through them, a few dynamic bodies that are triggers themselves (they
    fall through everything, the ground included) and a jointed capsule chain with a
    trigger link (a trigger pair is tested ahead of the jointed-pair filter)."""
    rng = scenes.SplitMix64(scenes.scene_seed(9, seed))
    s = scenes.SceneData("triggers%d" % seed)
    scenes._ground_box(s, (9.0, 0.5, 9.0))
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(9, 1 << 19)), count=4)
    s.convex.extend(pool)
    q = rng.quaternions(4)
    s.add_bodies(pos=[[0.0, 3.0, 0.0], [4.5, 1.5, 4.5], [-4.5, 1.5, -4.5], [4.5, 1.5, -4.5]], quat=q, flags=0,
                 inv_mass=0.0, com=np.zeros(3), inv_inertia=np.zeros(9),
                 col_type=[scenes.BOX, scenes.SPHERE, scenes.CAPSULE, scenes.CONVEX_MESH],
                 col_params=[[5.0, 0.4, 5.0, 0.0], [1.5, 0.0, 0.0, 0.0], [2.0, 0.6, 0.0, 0.0], [2.0, 2.0, 2.0, 0.0]],
                 col_mesh=[-1, -1, -1, 0])
    centers = scenes._jittered_grid(rng, 6, 3, 6, 1.5, [0.0, 6.0, 0.0])[:n]
    first = scenes._mixed_bodies(s, rng, centers, 0, pool)
    chain = scenes._chain(s, rng, 0, [0.0, -0.5, 0.0], [7.5, 6.0, 7.5], 6, [scenes.JOINT_SPHERICAL] * 6)
    s = s.finalize()
    trig = s.arrays["col_is_trigger"]
    trig[1:5] = 1
    trig[first + np.arange(3, n, 11)] = 1
    trig[chain + 2] = 1
    return s


def delta_schedule(s, frames, seed=5, every=3):
    """Seeded registry deltas for a scene: frame -> list of psx_body_delta dicts, every
    `every` frames.  Poses teleport bodies (static ones too) above the scene; velocities
    kick dynamic bodies; kinematic flags toggle on dynamic bodies, jointed ones included
    (bodies jointed in the overflow colour are left alone); one body per batch gets a
    velocity, a kinematic toggle and a second velocity in that order, so that the fold of
    a batch matters."""
    a = s.arrays
    rng = np.random.default_rng(seed)
    nb = len(a["pos"])
    dyn = np.nonzero(a["flags"] & scenes.BODY_DYNAMIC)[0]
    # bodies in a joint colour past the eighth (the reference's greedy bitset colouring)
    bits = np.zeros(nb, np.int64)
    overflow = set()
    for b0, b1 in zip(a.get("joint_body0", []), a.get("joint_body1", [])):
        u = bits[b0] | bits[b1]
        c = 0
        while u >> c & 1:
            c += 1
        if c >= 8:
            overflow.update((int(b0), int(b1)))
        bits[b0] |= 1 << c
        bits[b1] |= 1 << c
    togglable = np.array([b for b in dyn if b not in overflow])
    kin = {int(b): bool(a["flags"][b] & scenes.BODY_KINEMATIC) for b in dyn}
    lo, hi = a["pos"].min(0), a["pos"].max(0)
    out = {}
    for f in range(0, frames, every):
        batch = []
        for b in rng.choice(nb, 2, replace=False):
            p = [rng.uniform(lo[0], hi[0]), hi[1] + rng.uniform(2, 5), rng.uniform(lo[2], hi[2])]
            q = rng.normal(size=4)
            batch.append({"body": int(b), "pos": np.float32(p), "quat": np.float32(q / np.linalg.norm(q))})
        for b in rng.choice(dyn, 2, replace=False):
            batch.append({"body": int(b), "vel": np.float32(rng.normal(0, 2, 3)), "ang_vel": np.float32(rng.normal(0, 1, 3))})
        if len(togglable):
            b = int(rng.choice(togglable))
            kin[b] = not kin[b]
            batch.append({"body": b, "kinematic": kin[b]})
            b = int(rng.choice(togglable))
            kin[b] = not kin[b]
            batch.append({"body": b, "vel": np.float32([0, 3, 0]), "ang_vel": np.float32([0, 0, 1])})
            batch.append({"body": b, "kinematic": kin[b]})
            batch.append({"body": b, "vel": np.float32(rng.normal(0, 1, 3)), "ang_vel": np.float32([0, 0, 0])})
        out[f] = batch
    return out


def spawn_body(rng, center, kind=None):
    """A single dynamic body (sphere, box or capsule) as a SceneData, for creating an
    entity after the scene's creation."""
    s = scenes.SceneData("spawn")
    kind = int(rng.integers(0, 3)) if kind is None else kind
    if kind == 0:
        r = float(rng.uniform(0.2, 0.5))
        m, com, inertia = scenes.mass_sphere(r)
        typ, prm = scenes.SPHERE, [r, 0, 0, 0]
    elif kind == 1:
        he = rng.uniform(0.15, 0.4, 3)
        m, com, inertia = scenes.mass_box(he)
        typ, prm = scenes.BOX, list(he) + [0]
    else:
        hh, r = float(rng.uniform(0.2, 0.5)), float(rng.uniform(0.15, 0.3))
        m, com, inertia = scenes.mass_capsule(hh, r)
        typ, prm = scenes.CAPSULE, [hh, r, 0, 0]
    q = rng.normal(size=4)
    s.add_bodies(pos=[center], quat=[q / np.linalg.norm(q)], flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m, com=com,
                 inv_inertia=np.linalg.inv(inertia).T.ravel(), col_type=typ, col_params=prm,
                 vel=[rng.normal(0, 1, 3)])
    return s.finalize()


def topology_schedule(s, frames, seed=7, every=4):
    """frame -> (bodies to destroy, SceneData bodies to create): every `every` frames two
    bodies that carry no joint (never the ground, body 0) are destroyed, also ones created
    earlier, and two or three bodies are dropped in above the scene."""
    a = s.arrays
    rng = np.random.default_rng(seed)
    jointed = set(np.asarray(a.get("joint_body0", []), int)) | set(np.asarray(a.get("joint_body1", []), int))
    alive = [b for b in range(1, len(a["pos"])) if b not in jointed]
    n = len(a["pos"])
    lo, hi = a["pos"].min(0), a["pos"].max(0)
    out = {}
    for f in range(0, frames, every):
        kill = [int(x) for x in rng.choice(alive, 2, replace=False)]
        for b in kill:
            alive.remove(b)
        spawn = []
        for _ in range(int(rng.integers(2, 4))):
            c = [rng.uniform(lo[0], hi[0]), hi[1] + rng.uniform(1, 3), rng.uniform(lo[2], hi[2])]
            spawn.append(spawn_body(rng, c))
            alive.append(n)
            n += 1
        out[f] = (kill, spawn)
    return out


def mechanism_scene(seed=71):
    """Every joint kind with its drive or parameters, beside free bodies that each touch
    only the ground.  No dynamic body carries two contacts, and joints are solved in the
    reference's own joint colours, so the frames do not depend on the order in which
    contacts are solved: the reference itself, run on the same registry, is the checker.
      - free bodies: 4 boxes, 4 spheres, 4 capsules and 4 hulls on a 4 m grid, dropped from
        1-2 m with seeded orientations and velocities, on a static ground box;
      - mechanisms under colliderless static anchors 8 m up, 3 m apart: a driven revolute
        link (RevoluteJoint drive, src/Joints/RevoluteJoint.cpp:30-37, 55); a prismatic
        link with limits and a drive (PrismaticJoint.cpp:81-97, 147-148); a servo link
        (ServoJoint.cpp:52-54); two revolute wheels coupled by a gear joint, one of them
        driven (GearJoint.cpp:10-57); spherical, universal and fixed two-link chains.
    Returns (scene, info) with the indices of the free bodies and of the joints by role."""
    rng = scenes.SplitMix64(scenes.scene_seed(11, seed))
    s = scenes.SceneData("mechanisms%d" % seed)
    scenes._ground_box(s, (20.0, 0.5, 20.0))
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(11, 1 << 19)), count=4)
    s.convex.extend(pool)
    g = (np.arange(4) - 1.5) * 4.0
    xs, zs = np.meshgrid(g, g, indexing="ij")
    centers = np.stack([xs.ravel(), 1.0 + rng.uniform(16), zs.ravel()], axis=1)
    kinds = np.repeat([scenes.BOX, scenes.SPHERE, scenes.CAPSULE, scenes.CONVEX_MESH], 4)
    free = []
    for i, c in enumerate(centers):
        mix = [0.0, 0.0, 0.0, 0.0]
        mix[[scenes.BOX, scenes.SPHERE, scenes.CAPSULE, scenes.CONVEX_MESH].index(kinds[i])] = 1.0
        first = scenes._mixed_bodies(s, rng, c[None, :], 0, pool, mix=tuple(mix))
        free.append(first)
    a_vel = rng.normal(3 * len(free)).reshape(-1, 3) * 0.5
    hh, r = 0.25, 0.1
    m, com, inertia = scenes.mass_capsule(hh, r)
    inv_i = np.linalg.inv(inertia).T.ravel()
    anchors = [[x, 8.0, 12.0] for x in np.arange(8) * 3.0 - 10.5]
    first_anchor = s.add_bodies(pos=anchors, quat=[scenes.IDENTITY_Q] * len(anchors), flags=0, inv_mass=0.0,
                                com=np.zeros(3), inv_inertia=np.zeros(9), col_type=scenes.SPHERE,
                                col_params=[0.1, 0, 0, 0])

    def link(at):
        return s.add_bodies(pos=[at], quat=[scenes.IDENTITY_Q], flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m, com=com,
                            inv_inertia=inv_i, col_type=scenes.CAPSULE, col_params=[hh, r, 0.0, 0.0])

    joints = []   # (kind, body0, body1, frames, params)
    roles = {}
    half = hh + r

    def hang(anchor, kind, params=None, links=1, q=scenes.IDENTITY_Q):
        top = np.asarray(anchors[anchor - first_anchor])
        prev, prev_off = anchor, [0.0, 0.0, 0.0]
        ids = []
        for k in range(links):
            b = link(top - [0.0, half + 2 * half * k, 0.0])
            joints.append((kind, prev, b, list(prev_off) + list(q) + [0.0, half, 0.0] + list(q),
                           params if params is not None else [0.0] * 8))
            ids.append(len(joints) - 1)
            prev, prev_off = b, [0.0, -half, 0.0]
        return ids

    qz = [0.0, 0.0, np.sin(np.pi / 4), np.cos(np.pi / 4)]   # anchor x axis along world y: a vertical slide
    roles["revolute_drive"] = hang(first_anchor + 0, scenes.JOINT_REVOLUTE, [1.0, 2.0, 50.0] + [0.0] * 5)
    roles["prismatic"] = hang(first_anchor + 1, scenes.JOINT_PRISMATIC, [0.2, -0.2, 1.0, 0.1, 5.0, 1.0, 0.0, 0.0], q=qz)
    roles["servo"] = hang(first_anchor + 2, scenes.JOINT_SERVO, [0.5, 30.0, 1.0] + [0.0] * 5)
    roles["spherical"] = hang(first_anchor + 3, scenes.JOINT_SPHERICAL, links=2)
    roles["universal"] = hang(first_anchor + 4, scenes.JOINT_UNIVERSAL, links=2)
    roles["fixed"] = hang(first_anchor + 5, scenes.JOINT_FIXED, links=2)
    # gear: two wheels on revolute joints under anchors 6 and 7, the first one driven.  The
    # axes run along world z, across the line between the wheels: the gear's angles are
    # measured from the direction between its anchors, which must not lie on the axis
    qy = [0.0, -np.sin(np.pi / 4), 0.0, np.cos(np.pi / 4)]   # anchor x axis along world z
    wa = roles["wheel_a"] = hang(first_anchor + 6, scenes.JOINT_REVOLUTE, [1.0, 1.5, 20.0] + [0.0] * 5, q=qy)
    wb = roles["wheel_b"] = hang(first_anchor + 7, scenes.JOINT_REVOLUTE, q=qy)
    ba, bb = joints[wa[0]][2], joints[wb[0]][2]
    joints.append((scenes.JOINT_GEAR, ba, bb, [0.0] * 3 + qy + [0.0] * 3 + qy, [2.0] + [0.0] * 7))
    roles["gear"] = [len(joints) - 1]
    s.add_joints(np.array([j[0] for j in joints], np.int32), np.array([j[1] for j in joints], np.int32),
                 np.array([j[2] for j in joints], np.int32), np.array([j[3] for j in joints]),
                 np.array([j[4] for j in joints]))
    s = s.finalize()
    s.arrays["ang_vel"][free] = a_vel.astype(np.float32)
    s = strip_colliders(s, range(first_anchor, first_anchor + len(anchors)))
    return s, {"free": free, "joints": roles}


OP_KINEMATIC, OP_PATCH, OP_JOINT, OP_VELOCITY = 1, 2, 3, 4


def mechanism_ops(s, info):
    """Registry edits between frames of mechanism_scene: (frame, op, index, values), applied
    before the frame: joint setters (a revolute drive reversed, new servo and prismatic
    targets, a new gear ratio), setIsKinematic on and off, a patched pose and directly
    written velocities."""
    free, j = info["free"], info["joints"]
    p = s.arrays["pos"][free[5]]
    return [
        (20, OP_JOINT, j["revolute_drive"][0], [1.0, -3.0, 50.0]),
        (25, OP_KINEMATIC, free[0], [1.0]),
        (30, OP_PATCH, free[5], [float(p[0]), 2.5, float(p[2]), 0.0, 0.0, 0.0, 1.0]),
        (35, OP_VELOCITY, free[3], [0.0, 3.0, 0.0, 0.0, 0.0, 1.0]),
        (40, OP_KINEMATIC, free[0], [0.0]),
        (45, OP_JOINT, j["servo"][0], [-0.5, 30.0, 1.0]),
        (45, OP_JOINT, j["prismatic"][0], [0.2, -0.2, 1.0, -0.1, 5.0, 1.0]),
        (50, OP_JOINT, j["gear"][0], [0.5]),
        (55, OP_JOINT, j["wheel_a"][0], [0.0, 0.0, 0.0]),
    ]


def apply_mechanism_op(sim, op):
    """One mechanism_ops entry through an OracleScene / RefScene / World interface."""
    from physecs_gb300.api import pack_deltas
    _, kind, idx, v = op
    if kind == OP_JOINT:
        sim.set_joint_params(idx, v)
    elif kind == OP_KINEMATIC:
        sim.apply_deltas(pack_deltas([{"body": idx, "kinematic": bool(v[0])}]))
    elif kind == OP_PATCH:
        sim.apply_deltas(pack_deltas([{"body": idx, "pos": v[:3], "quat": v[3:7]}]))
    elif kind == OP_VELOCITY:
        sim.apply_deltas(pack_deltas([{"body": idx, "vel": v[:3], "ang_vel": v[3:6]}]))


def mechanism_topology_ops(s, info):
    """Topology edits of mechanism_scene for an application driving the registry
    (tests/shim/drive_scene.cpp op codes 5-9), each keeping every dynamic body to at
    most one contact: a free body destroyed, another's colliders cleared, a sphere
    collider added high above a third, a fixed and a universal joint destroyed,
    and a sphere entity created in a free spot."""
    free, j = info["free"], info["joints"]
    return [
        (15, 5, free[7], []),
        (18, 6, free[10], []),
        (22, 7, free[11], [0.2, 0.0, 1.8, 0.0]),
        (26, 8, j["fixed"][1], []),
        (28, 9, -1, [0.3, 8.0, 2.0, -8.0, 1.0 / 113.1, 1.0 / 4.07]),
        (33, 8, j["universal"][1], []),
    ]


def scattered_scene(seed=53, n_dense=480, n_clumps=160):
    """Bodies that are neighbours on the broadphase's Morton curve yet far apart: a dense
    block of mixed bodies on a ground box, and clumps of three overlapping bodies scattered
    over a 400 m cube.  Warps of the pair walk then take both coherent and scattered
    leaves (the second kind is walked one lane at a time)."""
    rng = scenes.SplitMix64(scenes.scene_seed(11, seed))
    s = scenes.SceneData("scattered%d" % seed)
    scenes._ground_box(s, (12.0, 0.5, 12.0))
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(11, 1 << 19)), count=4)
    s.convex.extend(pool)
    dense = scenes._jittered_grid(rng, 10, 5, 10, 1.5, [0.0, 1.5, 0.0])[:n_dense]
    far = rng.uniform(3 * n_clumps, -200.0, 200.0).reshape(n_clumps, 3)
    jitter = rng.uniform(9 * n_clumps, -0.4, 0.4).reshape(n_clumps, 3, 3)
    clumps = (far[:, None, :] + jitter).reshape(-1, 3)
    scenes._mixed_bodies(s, rng, np.concatenate([dense, clumps]), 0, pool)
    return s.finalize()
