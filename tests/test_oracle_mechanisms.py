"""Joint drives, limits, the servo and the gear in the CPU oracle, against the reference.

mechanism_scene holds every joint kind with the parameters round-one scenes never set:
a driven revolute joint (src/Joints/RevoluteJoint.cpp:30-37, 55), a prismatic joint with
limits and a drive (PrismaticJoint.cpp:81-97, 147-148), a servo (ServoJoint.cpp:52-54)
and a gear between two revolute wheels (GearJoint.cpp:10-57); between frames the joint
setters change drives, targets and the gear ratio, and the registry is edited.  The
oracle's body states equal the reference's bit for bit: against tests/golden/
mechanisms.npz (made by the reference, tests/golden/make_golden.py) and, where the
reference library is built here, live."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from scene_variants import apply_mechanism_op, mechanism_ops, mechanism_scene  # noqa: E402


def _run(sim, s, info, frames, record):
    ops = mechanism_ops(s, info)
    out = {}
    for f in range(frames):
        for op in ops:
            if op[0] == f:
                apply_mechanism_op(sim, op)
        sim.step()
        if f + 1 in record:
            out[f + 1] = sim.state()
    return out


def test_oracle_matches_reference_fixture(oracle_lib):
    from oracle.port_api import OracleScene
    d = np.load(os.path.join(HERE, "golden", "mechanisms.npz"))
    s, info = mechanism_scene()
    assert str(d["scene_sha256"]) == make_golden.scene_hash(s)
    got = _run(OracleScene(s), s, info, make_golden.MECHANISM_FRAMES, make_golden.MECHANISM_RECORDED)
    for f, st in got.items():
        for k, v in st.items():
            assert not np.isnan(v).any(), (f, k)
            assert np.array_equal(v.view(np.uint32), d["f%d_%s" % (f, k)].view(np.uint32)), (f, k)
    # the drives and the gear did something: the wheels turn, in opposite senses
    j = info["joints"]
    wa = s.arrays["joint_body1"][j["wheel_a"][0]]
    assert abs(d["f30_ang_vel"][wa]).max() > 1e-2


def test_oracle_matches_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import OracleScene
    from oracle.ref.ref_api import RefScene
    s, info = mechanism_scene(seed=72)
    rec = list(range(1, 91))
    a = _run(OracleScene(s), s, info, 90, rec)
    b = _run(RefScene(s), s, info, 90, rec)
    for f in rec:
        for k in a[f]:
            assert np.array_equal(a[f][k].view(np.uint32), b[f][k].view(np.uint32)), (f, k)
