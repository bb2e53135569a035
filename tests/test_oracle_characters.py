"""CharacterController::move (src/CharacterController.cpp:5-45) in the CPU oracle against
the reference's own controller, run side by side where the reference library is built:
the same flags and the same scene state bit for bit, frame after frame."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from scene_variants import character_moves, character_scene  # noqa: E402


def test_oracle_characters_match_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    for seed in (61, 63):
        s, chars = character_scene(seed)
        o, r = OracleScene(s), RefScene(s)
        moves = character_moves(len(chars), 40, seed=seed + 1)
        seen = 0
        for f in range(40):
            for k, b in enumerate(chars):
                fo = o.move_character(b, 1.0, 0.3, moves[f][k], iterations=2 + (k % 2))
                fr = r.move_character(b, 1.0, 0.3, moves[f][k], iterations=2 + (k % 2))
                assert fo == fr, (seed, f, k)
                seen |= fo
            o.step()
            r.step()
        so, sr = o.state(), r.state()
        for k in so:
            assert np.array_equal(so[k].view(np.uint32), sr[k].view(np.uint32)), (seed, k)
        assert seen == 7


def test_character_entity_without_colliders(oracle_lib):
    """A controller's entity holds a transform and no collider: its own capsule query
    never meets itself, and a frame leaves it where the controller put it."""
    from oracle.port_api import OracleScene
    s, chars = character_scene(n_chars=3)
    assert (np.diff(s.arrays["collider_start"])[chars] == 0).all()
    o = OracleScene(s)
    o.move_character(chars[0], 1.0, 0.3, [0.1, 0.0, 0.0])
    p = o.state()["pos"][chars[0]].copy()
    o.step()
    assert np.array_equal(o.state()["pos"][chars[0]], p)
