"""The triangle-mesh BVH built on the GPU (psx_trimesh_build, psx_world_update_trimesh)
against the reference's layout: triangles and nodes bit for bit against the golden
meshes (made by the reference, tests/golden/trimesh_bvh.npz) and against the oracle on
meshes large enough to run the level kernels (several chunks per node, deep trees,
leaves above the chunk size)."""
import os
import sys

import numpy as np
import pytest

from physecs_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _same_tris(a, b):
    """Triangle words equal bit for bit, except that a NaN (the normal of a zero-area
    triangle, normalize of a zero vector) only has to be NaN on both sides: the bits of a
    NaN that an operation creates differ between x86, Arm and CUDA."""
    if a.shape != b.shape:
        return False
    fa, fb = a[:, 4:].view(np.float32), b[:, 4:].view(np.float32)
    na, nb = np.isnan(fa), np.isnan(fb)
    return (np.array_equal(a[:, :4], b[:, :4]) and np.array_equal(na, nb)
            and np.array_equal(a[:, 4:][~na], b[:, 4:][~nb]))


@pytest.mark.parametrize("name", [n for n, (_, ix) in make_golden.trimesh_cases().items() if len(ix)])
def test_device_bvh_matches_reference_fixture(gpu_lib, name):
    from physecs_gb300.api import trimesh_build
    d = np.load(os.path.join(HERE, "golden", "trimesh_bvh.npz"))
    v, ix = make_golden.trimesh_cases()[name]
    tris, nodes = trimesh_build(v, ix)
    assert np.array_equal(nodes, d[name + "__nodes"])
    assert _same_tris(tris, d[name + "__tris"])


def test_device_bvh_of_an_empty_mesh(gpu_lib, oracle_lib):
    """One empty leaf, as the oracle's (the reference's constructor throws here)."""
    from oracle.port_api import trimesh_build as orc_build
    from physecs_gb300.api import trimesh_build
    v = np.zeros((3, 3), np.float32)
    t, n = trimesh_build(v, np.zeros(0, np.uint32))
    to, no = orc_build(v, np.zeros(0, np.uint32))
    assert len(t) == 0 and np.array_equal(n, no)


def _large_meshes():
    rng = np.random.default_rng(11)
    out = {}
    v, ix, _ = scenes.heightfield(scenes.SplitMix64(21), cells=256)
    out["heightfield256"] = (v, ix.ravel())
    n = 40000
    v = rng.normal(0, 20, (3 * n, 3)).astype(np.float32)
    v[rng.random(3 * n) < 0.05] = 0.0
    ix = np.arange(3 * n, dtype=np.uint32)
    ix = np.concatenate([ix, ix.reshape(-1, 3)[rng.integers(0, n, 4000)].ravel()])   # duplicates: shared leaves
    out["soup40k"] = (v, ix)
    k = np.arange(3000)
    x = (1.01 ** k).astype(np.float32)
    z0 = np.zeros_like(x)
    v = np.stack([np.stack([x, z0, z0], 1), np.stack([x + 0.5, z0 + 1, z0], 1), np.stack([x, z0, z0 + 1], 1)], 1)
    out["skewed3000"] = (v.reshape(-1, 3).astype(np.float32),
                         (rng.permutation(3000).repeat(3) * 3 + np.tile(np.arange(3), 3000)).astype(np.uint32))
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [5, 5, 5], [6, 5, 5], [5, 5, 6]], np.float32)
    same = np.tile(np.array([0, 1, 2], np.uint32), 5000)
    out["shared_centroids"] = (v, np.concatenate([same, np.tile(np.array([3, 4, 5], np.uint32), 3000)]))
    return out


@pytest.mark.parametrize("name", list(_large_meshes()))
def test_device_bvh_matches_oracle_on_large_meshes(gpu_lib, oracle_lib, name):
    from oracle.port_api import trimesh_build as orc_build
    from physecs_gb300.api import trimesh_build
    v, ix = _large_meshes()[name]
    t, n = trimesh_build(v, ix)
    to, no = orc_build(v, ix)
    assert len(n) == len(no)
    assert np.array_equal(n, no)
    assert _same_tris(t, to)


def test_world_update_trimesh(gpu_lib):
    """A world whose heightfield is replaced before it steps behaves bit for bit as a world
    created with the new heightfield: the same bounds, the same states frame by frame."""
    from physecs_gb300.api import World
    s1 = scenes.large_mixed(n_bodies=200, cells=32, seed=5)
    s2 = scenes.large_mixed(n_bodies=200, cells=32, seed=5)
    a2 = s2.arrays
    m0, m1 = a2["tri_vert_start"][0], a2["tri_vert_start"][1]
    new = a2["tri_verts"][m0:m1].copy()
    new[:, 1] = new[:, 1] * np.float32(0.5) + np.float32(0.25)
    a2["tri_verts"][m0:m1] = new
    wa, wb = World([s1, s1]), World([s1, s2])
    wa.update_trimesh(1, 0, new)
    assert np.array_equal(wa.bounds().view(np.uint32), wb.bounds().view(np.uint32))
    for _ in range(20):
        wa.step()
        wb.step()
    sa, sb = wa.read_bodies(), wb.read_bodies()
    for k in sa:
        assert np.array_equal(sa[k].view(np.uint32), sb[k].view(np.uint32)), k
    assert wa.counts()["error"] == 0
    # the scene that kept its mesh is untouched by the other's update
    wc = World([s1])
    for _ in range(20):
        wc.step()
    n0 = len(s1.arrays["pos"])
    assert np.array_equal(sa["pos"][:n0].view(np.uint32), wc.read_bodies()["pos"].view(np.uint32))
