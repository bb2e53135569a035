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
