"""Joint drives, limits, the servo and the gear on the GPU, against the oracle.

mechanism_scene (tests/scene_variants.py) with its registry edits between frames, the
joint setters among them (psx_world_set_joint_params), run in lockstep with the oracle
fed the GPU's contact order: every frame's body state within 1e-5 relative, and the
recorded frames against the reference's fixture (tests/golden/mechanisms.npz) within the
same tolerance.  The servo and gear rows call the device's acosf / atan2f / fmodf where
the reference calls the host's; the observed difference is reported by the assertion
message if it ever exceeds the tolerance."""
import os
import sys

import numpy as np
import pytest

from tests.parity import gpu_keys, rel_state_diff

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from scene_variants import apply_mechanism_op, mechanism_ops, mechanism_scene  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.mark.parametrize("seed", [71, 72])
def test_mechanisms_in_lockstep_with_oracle(gpu_lib, oracle_lib, seed):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    s, info = mechanism_scene(seed=seed)
    ops = mechanism_ops(s, info)
    g = World([s], use_graph=True)
    o = OracleScene(s)
    d = np.load(os.path.join(HERE, "golden", "mechanisms.npz")) if seed == 71 else None
    worst = 0.0
    for f in range(make_golden.MECHANISM_FRAMES):
        for op in ops:
            if op[0] == f:
                apply_mechanism_op(g, op)
                apply_mechanism_op(o, op)
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0, f
        st = g.read_bodies()
        diff = rel_state_diff(st, o.state())
        worst = max(worst, diff)
        assert diff <= TOL, "frame %d: relative state difference %g" % (f + 1, diff)
        if d is not None and f + 1 in make_golden.MECHANISM_RECORDED:
            ref = {k: d["f%d_%s" % (f + 1, k)] for k in ("pos", "quat", "vel", "ang_vel")}
            r = rel_state_diff(st, ref)
            assert r <= TOL, "frame %d: %g from the reference's fixture" % (f + 1, r)
    assert g.counts()["error"] == 0
    print("largest relative difference over %d frames: %g" % (make_golden.MECHANISM_FRAMES, worst))
