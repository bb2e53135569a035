"""The C++ drop-in (include/physecs_gb300/Physecs.h) on CPU.

One Physecs application source (tests/shim/drive_scene.cpp) compiles both against the
reference's own headers and library and against the drop-in header with libpsx.so, with
g++, EnTT and GLM as vendored by the reference.  The registry components it reads have
the reference's layout.  Run on this machine's CPU, the reference build reproduces the
oracle, and the drop-in build fails loudly for want of a GPU instead of falling back."""
import os
import subprocess

import numpy as np
import pytest

from tests.scene_variants import mechanism_ops, mechanism_scene

LAYOUT = {
    "TransformComponent": 40, "TransformComponent.position": 0, "TransformComponent.orientation": 12,
    "TransformComponent.scale": 28,
    "RigidBodyDynamicComponent": 80, "RigidBodyDynamicComponent.isKinematic": 0,
    "RigidBodyDynamicComponent.velocity": 4, "RigidBodyDynamicComponent.angularVelocity": 16,
    "RigidBodyDynamicComponent.invMass": 28, "RigidBodyDynamicComponent.com": 32,
    "RigidBodyDynamicComponent.invInertiaTensor": 44,
    "RigidBodyCollisionComponent": 24,
    "Collider": 88, "Collider.position": 0, "Collider.orientation": 12, "Collider.geometry": 32,
    "Collider.material": 64, "Collider.isTrigger": 76, "Collider.enableSimulation": 77, "Collider.data": 80,
    "Geometry": 32, "quat.x": 1, "quat.storage0": 1, "quat.storage3": 4,
}


def _tree_or_skip():
    from oracle.ref import build_ref
    if not os.path.isdir(build_ref.TREE):
        pytest.skip("no copy of the reference's headers (oracle/ref/build_ref.py makes one)")


def test_component_layouts_as_the_reference_headers_give_them():
    _tree_or_skip()
    from tests.shim import scene_file as sf
    out = subprocess.run([sf.build_layout_check()], capture_output=True, text=True, check=True).stdout
    got = {k: int(v) for k, v in (line.split() for line in out.splitlines())}
    assert got == LAYOUT


def test_one_application_builds_against_both(tmp_path):
    _tree_or_skip()
    from oracle.ref import ref_api
    from oracle.port_api import OracleScene
    from tests.shim import scene_file as sf
    from tests.scene_variants import apply_mechanism_op
    shim = sf.build_shim()
    s, info = mechanism_scene()
    ops = mechanism_ops(s, info)
    path = str(tmp_path / "mech.scene")
    sf.write_scene(path, s, 40, ops)
    n = len(s.arrays["pos"])
    if ref_api.available():
        rc, err, st = sf.run(sf.build_reference(), path, str(tmp_path / "ref.out"), n, 40)
        assert rc == 0, err
        o = OracleScene(s)
        for f in range(40):
            for op in ops:
                if op[0] == f:
                    apply_mechanism_op(o, op)
            o.step()
            got = o.state()
            want = np.concatenate([got["pos"], got["quat"], got["vel"], got["ang_vel"]], 1)
            assert np.array_equal(want.view(np.uint32), st[f].view(np.uint32)), f
    import torch
    if not torch.cuda.is_available():
        rc, err, _ = sf.run(shim, path, str(tmp_path / "shim.out"), n, 40)
        assert rc == 2 and "physecs_gb300" in err, (rc, err)
