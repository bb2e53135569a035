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
