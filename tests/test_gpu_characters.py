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
