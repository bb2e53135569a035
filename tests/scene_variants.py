"""Scenes that exercise the reference's less common inputs: kinematic bodies (moving,
never integrated), trigger colliders (no contacts), colliders with enableSimulation
off (no pairs), a scene without dynamic bodies and a scene without any contact."""
import numpy as np

from physecs_gb300 import scenes


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


def strip_colliders(s, bodies):
    """The scene with the colliders of `bodies` removed: such a body is an entity with a
    transform and an empty collider list (a character controller's entity)."""
    a = s.arrays
    cs = a["collider_start"]
    keep = np.ones(cs[-1], bool)
    for b in bodies:
        keep[cs[b]:cs[b + 1]] = False
    per_body = np.diff(cs).copy()
    per_body[list(bodies)] = 0
    for k in list(a):
        if k.startswith("col_") and len(a[k]) == len(keep):
            a[k] = np.ascontiguousarray(a[k][keep])
    a["collider_start"] = np.concatenate([[0], np.cumsum(per_body)]).astype(np.int32)
    return s


def character_scene(seed=61, n_chars=24, n_balls=10):
    """Character entities (transforms without colliders) among static walls, a ramp and
    resting dynamic bodies on a ground box."""
    rng = np.random.default_rng(seed)
    s = scenes.SceneData("characters%d" % seed)
    scenes._ground_box(s, (12.0, 0.5, 12.0))
    walls = [([0, 1, 6], [6, 1, 0.3]), ([6, 1, 0], [0.3, 1, 6]), ([-4, 0.5, -4], [1.5, 0.5, 1.5])]
    for p, he in walls:
        s.add_bodies(pos=[p], quat=[scenes.IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3), inv_inertia=np.zeros(9),
                     col_type=scenes.BOX, col_params=list(he) + [0.0])
    ang = 0.35
    s.add_bodies(pos=[[-3, 0.6, 3]], quat=[[np.sin(ang / 2), 0, 0, np.cos(ang / 2)]], flags=0, inv_mass=0.0,
                 com=np.zeros(3), inv_inertia=np.zeros(9), col_type=scenes.BOX, col_params=[2, 0.2, 2, 0])
    m, com, inertia = scenes.mass_sphere(0.4)
    balls = rng.uniform(-5, 5, (n_balls, 3))
    balls[:, 1] = 0.4 + 0.9 * (np.arange(n_balls) // 10)
    s.add_bodies(pos=balls, quat=[scenes.IDENTITY_Q] * n_balls, flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m, com=com,
                 inv_inertia=np.linalg.inv(inertia).T.ravel(), col_type=scenes.SPHERE, col_params=[0.4, 0, 0, 0])
    pc = rng.uniform(-6, 6, (n_chars, 3))
    pc[:, 1] = rng.uniform(0.0, 0.3, n_chars)
    first = s.add_bodies(pos=pc, quat=[scenes.IDENTITY_Q] * n_chars, flags=0, inv_mass=0.0, com=np.zeros(3),
                         inv_inertia=np.zeros(9), col_type=scenes.SPHERE, col_params=[0.1, 0, 0, 0])
    s = s.finalize()
    return strip_colliders(s, range(first, first + n_chars)), list(range(first, first + n_chars))


def character_moves(n_chars, frames, seed=62):
    """Seeded translations per frame and character: a walk in a heading that turns, plus a
    downward pull."""
    rng = np.random.default_rng(seed)
    head = rng.uniform(0, 2 * np.pi, n_chars)
    out = []
    for _ in range(frames):
        head += rng.normal(0, 0.3, n_chars)
        t = np.stack([0.12 * np.cos(head), np.full(n_chars, -0.05), 0.12 * np.sin(head)], 1).astype(np.float32)
        out.append(t)
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
