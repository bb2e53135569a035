"""The triangle-mesh BVH of the CPU oracle (TriangleMesh's constructor, binned SAH,
src/TriangleMesh.cpp:7-164) against the reference: triangles and nodes bit for bit on
the golden meshes of tests/golden/trimesh_bvh.npz (made by the reference,
tests/golden/make_golden.py) and, where the reference library is built, on larger
seeded meshes side by side."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

FIX = os.path.join(HERE, "golden", "trimesh_bvh.npz")


@pytest.mark.parametrize("name", [n for n, (_, ix) in make_golden.trimesh_cases().items() if len(ix)])
def test_oracle_bvh_matches_reference_fixture(oracle_lib, name):
    from oracle.port_api import trimesh_build
    d = np.load(FIX)
    v, ix = make_golden.trimesh_cases()[name]
    assert np.array_equal(d[name + "__verts"].view(np.uint32), v.view(np.uint32))
    assert np.array_equal(d[name + "__indices"], ix)
    tris, nodes = trimesh_build(v, ix)
    assert np.array_equal(nodes, d[name + "__nodes"])
    # NaN normals of zero-area triangles carry the platform's default NaN bits
    ft, fd = tris[:, 4:].view(np.float32), d[name + "__tris"][:, 4:].view(np.float32)
    assert np.array_equal(np.isnan(ft), np.isnan(fd))
    assert np.array_equal(tris[:, :4], d[name + "__tris"][:, :4])
    assert np.array_equal(tris[:, 4:][~np.isnan(ft)], d[name + "__tris"][:, 4:][~np.isnan(fd)])


def test_bvh_structure(oracle_lib):
    """Every triangle sits in exactly one leaf; an inner node's children are index and
    index + 1; the cases reach their intended branches (a leaf that no split divides,
    leaves of several triangles, a single-triangle root)."""
    d = np.load(FIX)
    for name, (_, ix) in make_golden.trimesh_cases().items():
        if not len(ix):
            continue
        nodes = d[name + "__nodes"]
        cnt, idx = nodes[:, 3].astype(np.int64), nodes[:, 7].astype(np.int64)
        covered = np.zeros(len(ix) // 3, np.int64)
        for c, i in zip(cnt, idx):
            if c:
                covered[i:i + c] += 1
        assert (covered == 1).all(), name
        inner = cnt == 0
        assert (idx[inner] + 1 < len(nodes)).all() and len(nodes) == 2 * int((~inner).sum()) - 1, name
    assert d["same_centroid__nodes"][0, 3] == 90
    assert d["soup__nodes"][:, 3].max() > 1
    assert len(d["single__nodes"]) == 1


def test_oracle_bvh_matches_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.port_api import trimesh_build
    from physecs_gb300 import scenes
    for seed, cells in ((3, 48), (4, 64)):
        v, ix, _ = scenes.heightfield(scenes.SplitMix64(seed), cells=cells)
        a = trimesh_build(v, ix.ravel())
        b = ref_api.trimesh_build(v, ix.ravel())
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])   # no zero-area triangle here
    # the reference's constructor throws for a mesh without triangles
    with pytest.raises(RuntimeError):
        ref_api.trimesh_build(np.zeros((3, 3), np.float32), np.zeros(0, np.uint32))
