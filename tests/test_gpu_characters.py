"""Character controllers on the GPU (psx_world_move_characters) against the oracle's
CharacterController::move: a batch of controllers moved every frame of a scene stepped in
lockstep (the oracle fed the GPU's contact order) gives the same flags and the same
states bit for bit.  The oracle's controller equals the reference's
(tests/test_oracle_characters.py)."""
import os
import sys

import numpy as np
import pytest

from tests.parity import gpu_keys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from scene_variants import character_moves, character_scene  # noqa: E402

pytestmark = pytest.mark.gpu


def test_characters_match_oracle(gpu_lib, oracle_lib):
    from oracle.port_api import OracleScene
    from physecs_gb300 import scenes
    from physecs_gb300.api import World
    s, chars = character_scene()
    other = scenes.batch_scene(5, n_bodies=40)
    g = World([other, s])
    o = OracleScene(s)
    moves = character_moves(len(chars), 40)
    seen = 0
    for f in range(40):
        specs = [{"scene": 1, "body": b, "height": 1.0, "radius": 0.3} for b in chars]
        fg = g.move_characters(specs, moves[f])
        fo = [o.move_character(b, 1.0, 0.3, moves[f][k]) for k, b in enumerate(chars)]
        assert list(fg) == fo, f
        seen |= int(np.bitwise_or.reduce(fg))
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        sel = ids[:, 0] == 1
        o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
        o.step()
        assert o.order_error() == 0
        st, so = g.read_bodies(), o.state()
        sl = slice(g.body_start[1], g.body_start[2])
        for k in so:
            assert np.array_equal(st[k][sl].view(np.uint32), so[k].view(np.uint32)), (f, k)
    assert seen == 7   # down, sides and up contacts all occurred
    assert g.counts()["error"] == 0


def test_character_refusals(gpu_lib):
    from physecs_gb300.api import PsxError, World
    s, chars = character_scene(n_chars=2)
    w = World([s])
    with pytest.raises(PsxError):
        w.move_characters([{"body": chars[0], "height": 1, "radius": 0.3}] * 2, np.zeros((2, 3)))
    with pytest.raises(PsxError):
        w.move_characters([{"scene": 1, "body": 0, "height": 1, "radius": 0.3}], np.zeros((1, 3)))
    assert len(w.move_characters([], np.zeros((0, 3)))) == 0


def test_controllers_that_meet_move_against_the_poses_before_the_batch(gpu_lib, oracle_lib):
    """Two controllers whose entities carry colliders, each within the other's reach: a
    batch moves both against the world as it was before the batch (neither sees the
    other's new pose), the same on every run, so each equals the oracle moving that
    controller alone from the poses before the batch."""
    from oracle.port_api import OracleScene
    from physecs_gb300 import scenes
    from physecs_gb300.api import World
    s = scenes.SceneData("meeting_controllers")
    scenes._ground_box(s, (5.0, 0.5, 5.0))
    # each entity's sphere sits beside the other controller's capsule, clear of its own
    s.add_bodies(pos=[[0.0, 0.05, 0.0], [0.9, 0.05, 0.0]], quat=[scenes.IDENTITY_Q] * 2, flags=0, inv_mass=0.0,
                 com=np.zeros(3), inv_inertia=np.zeros(9), col_type=scenes.SPHERE, col_params=[0.2, 0.0, 0.0, 0.0],
                 col_pos=[[0.6, 0.8, 0.0], [-0.6, 0.8, 0.0]])
    s = s.finalize()
    chars = [1, 2]
    moves = np.array([[0.2, -0.05, 0.0], [-0.2, -0.05, 0.0]], np.float32)
    specs = [{"body": b, "height": 1.0, "radius": 0.3} for b in chars]
    runs = []
    for _ in range(3):
        g = World([s])
        flags = g.move_characters(specs, moves)
        runs.append((list(flags), g.read_bodies()["pos"][chars].copy()))
        assert g.counts()["error"] == 0
        g.close()
    for r in runs[1:]:
        assert r[0] == runs[0][0] and np.array_equal(r[1], runs[0][1])
    for k, b in enumerate(chars):
        o = OracleScene(s)
        fo = o.move_character(b, 1.0, 0.3, moves[k])
        assert fo == runs[0][0][k], k
        assert np.array_equal(o.state()["pos"][b].view(np.uint32), runs[0][1][k].view(np.uint32)), k
    assert runs[0][0][0] & 2 and runs[0][0][1] & 2   # each met the other at its side
