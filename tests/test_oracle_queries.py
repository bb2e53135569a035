"""Scene queries of the CPU oracle (Scene::raycastClosest, Scene::overlap) against the
reference: the golden answers in tests/golden/queries.npz, made by the reference from
its own sources (tests/golden/make_golden.py), and, where the reference library is
built, fresh seeded queries side by side."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

FIX = os.path.join(HERE, "golden", "queries.npz")


def _fixture():
    return np.load(FIX)


def _stepped_oracle(s, frames):
    from oracle.port_api import OracleScene
    o = OracleScene(s)
    for _ in range(frames):
        o.step()
    return o


def _overlaps(sim, d, pre):
    out = []
    for k in range(len(d[pre + "q_type"])):
        out.append(sorted(sim.overlap(d[pre + "q_pos"][k], d[pre + "q_quat"][k], d[pre + "q_type"][k],
                                      d[pre + "q_params"][k], d[pre + "q_mesh"][k], d[pre + "q_filter"][k])))
    return out


@pytest.mark.parametrize("name", list(make_golden.query_scenes()))
def test_oracle_queries_match_reference_fixture(oracle_lib, name):
    d = _fixture()
    s, frames = make_golden.query_scenes()[name]
    pre = name + "__"
    assert str(d[pre + "scene_sha256"]) == make_golden.scene_hash(s)
    o = _stepped_oracle(s, frames)
    h = o.raycast(d[pre + "rays"], d[pre + "accept"])
    assert np.array_equal(h["body"], d[pre + "ray_body"])
    hit = h["body"] >= 0
    assert hit.sum() > 100
    assert np.array_equal(h["pos"][hit].view(np.uint32), d[pre + "ray_pos"][hit].view(np.uint32))
    got = _overlaps(o, d, pre)
    st, flat = d[pre + "q_start"], d[pre + "q_hits"]
    for k, g in enumerate(got):
        want = [tuple(map(int, r)) for r in flat[st[k]:st[k + 1]]]
        assert g == want, k
    assert st[-1] > 100
    ms, mids, mf = d[pre + "mtd_start"], d[pre + "mtd_ids"], d[pre + "mtd_f"]
    for k in range(len(d[pre + "q_type"])):
        got = make_golden.mtd_sorted(o.overlap_mtd(d[pre + "q_pos"][k], d[pre + "q_quat"][k], d[pre + "q_type"][k],
                                                   d[pre + "q_params"][k], d[pre + "q_mesh"][k]))
        assert [(b, c) for b, c, _, _ in got] == [tuple(map(int, r)) for r in mids[ms[k]:ms[k + 1]]], k
        gf = np.asarray([list(n) + [m] for _, _, n, m in got], np.float32).reshape(-1, 4)
        assert np.array_equal(gf.view(np.uint32), mf[ms[k]:ms[k + 1]].view(np.uint32)), k
    assert ms[-1] > 100


def test_reference_raycast_without_filter_never_hits():
    """The reference's raycastClosest overload without a filter tests an empty
    std::function, so it reports no hit whatever the ray (src/Physecs.cpp:580, 615)."""
    d = _fixture()
    for name in make_golden.query_scenes():
        assert (d[name + "__ray_body_nofilter"] == -1).all()
        assert (d[name + "__ray_body"] >= 0).any()


def test_oracle_queries_match_live_reference(oracle_lib):
    from oracle.ref import ref_api
    if not ref_api.available():
        pytest.skip("reference library not built here")
    from oracle.ref.ref_api import RefScene
    for si, (name, (s, frames)) in enumerate(make_golden.query_scenes().items()):
        o = _stepped_oracle(s, frames)
        r = RefScene(s)
        for _ in range(frames):
            r.step()
        rays, accept, qpos, qquat, kinds, prm, mesh, filt = make_golden.query_inputs(s, r.state()["pos"], 900 + si)
        ho, hr = o.raycast(rays, accept), r.raycast(rays, accept)
        assert np.array_equal(ho["body"], hr["body"]), name
        hit = hr["body"] >= 0
        assert np.array_equal(ho["pos"][hit].view(np.uint32), hr["pos"][hit].view(np.uint32)), name
        for k in range(len(kinds)):
            a = sorted(o.overlap(qpos[k], qquat[k], kinds[k], prm[k], mesh[k], filt[k]))
            b = sorted(r.overlap(qpos[k], qquat[k], kinds[k], prm[k], mesh[k], filt[k]))
            assert a == b, (name, k)
            a = make_golden.mtd_sorted(o.overlap_mtd(qpos[k], qquat[k], kinds[k], prm[k], mesh[k]))
            b = make_golden.mtd_sorted(r.overlap_mtd(qpos[k], qquat[k], kinds[k], prm[k], mesh[k]))
            assert [(x[0], x[1]) for x in a] == [(x[0], x[1]) for x in b], (name, k)
            fa = np.asarray([list(x[2]) + [x[3]] for x in a], np.float32).reshape(-1, 4)
            fb = np.asarray([list(x[2]) + [x[3]] for x in b], np.float32).reshape(-1, 4)
            assert np.array_equal(fa.view(np.uint32), fb.view(np.uint32)), (name, k)
