"""The C++ drop-in on the GPU: one Physecs application, two builds, the same frames.

tests/shim/drive_scene.cpp builds a registry through the reference's public API (entities,
components, meshes, createJoint<T> and the joint setters), edits it between frames
(setIsKinematic, registry.patch, direct velocity writes, joint setters) and calls
Scene::simulate.  Built against the reference's headers and library it runs the
reference's CPU code; built against include/physecs_gb300/Physecs.h it runs on this GPU
through libpsx.so.  mechanism_scene keeps every dynamic body to one contact, so the
reference's serial contact order and the GPU's colour order give the same frames: every
frame's registry state agrees within 1e-5 relative, also across topology changes
(entities destroyed and created, colliders cleared and added, joints destroyed)."""
import numpy as np
import pytest

from tests.scene_variants import mechanism_ops, mechanism_scene, mechanism_topology_ops

pytestmark = pytest.mark.gpu

TOL = 1e-5
FRAMES = 120


def _rel(a, b):
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b)
    a, b = a[~nan_a].astype(np.float64), b[~nan_b].astype(np.float64)
    return float((np.abs(a - b) / np.maximum(1.0, np.abs(b))).max()) if a.size else 0.0


@pytest.mark.parametrize("seed,topology", [(71, False), (73, False), (71, True)])
def test_application_on_the_drop_in_equals_the_reference(gpu_lib, tmp_path, seed, topology):
    """With topology=True the application also destroys an entity, clears one entity's
    colliders, adds a collider to another, destroys two joints and creates an entity
    between frames (the drop-in rebuilds its device world with psx_world_recreate)."""
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from tests.shim import scene_file as sf
    s, info = mechanism_scene(seed=seed)
    path = str(tmp_path / "scene")
    ops = mechanism_ops(s, info) + (mechanism_topology_ops(s, info) if topology else [])
    sf.write_scene(path, s, FRAMES, ops)
    n = len(s.arrays["pos"]) + sum(1 for o in ops if o[1] == sf.OP_SPAWN_SPHERE)
    rc, err, ref = sf.run(sf.build_reference(), path, str(tmp_path / "ref.out"), n, FRAMES)
    assert rc == 0, err
    rc, err, gpu = sf.run(sf.build_shim(), path, str(tmp_path / "gpu.out"), n, FRAMES)
    assert rc == 0, err
    for f in range(FRAMES):
        d = _rel(gpu[f], ref[f])
        assert d <= TOL, "frame %d: relative difference %g" % (f + 1, d)
    # the scene moved: bodies fell onto the ground and the mechanisms turned
    assert np.abs(ref[-1][:, :3] - ref[0][:, :3]).max() > 0.1
