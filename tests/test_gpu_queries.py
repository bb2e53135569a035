"""Scene queries on the GPU (psx_world_raycast, psx_world_overlap) against the oracle.

The GPU world and the oracle run in lockstep (the oracle fed the GPU's contact order),
so both hold the same state and bounds; the queries of tests/golden/queries.npz then
give the same closest hit (body, collider, distance and position, bit for bit) and the
same overlap sets.  The oracle's answers equal the reference's (tests/test_oracle_queries.py)."""
import os
import sys

import numpy as np
import pytest

from physecs_gb300 import scenes
from tests.parity import gpu_keys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _lockstep(ss, frames):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    g = World(ss)
    os_ = [OracleScene(s) for s in ss]
    for _ in range(frames):
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        for i, o in enumerate(os_):
            sel = ids[:, 0] == i
            o.set_contact_order(gpu_keys(ids[sel], meta[sel]))
            o.step()
            assert o.order_error() == 0
    return g, os_


def _queries(d, pre, scene):
    qs = []
    for k in range(len(d[pre + "q_type"])):
        qs.append({"scene": scene, "pos": d[pre + "q_pos"][k], "quat": d[pre + "q_quat"][k], "type": int(d[pre + "q_type"][k]),
                   "params": d[pre + "q_params"][k], "mesh": int(d[pre + "q_mesh"][k]), "filter": int(d[pre + "q_filter"][k])})
    return qs


def _check_scene(g, o, d, pre, scene, body0, nbodies_world, min_hits=50):
    rays = d[pre + "rays"].astype(np.float64).copy()
    rays[:, 0] = scene
    acc = d[pre + "accept"]
    acc_world = np.ones(nbodies_world, np.uint8)
    acc_world[body0:body0 + len(acc)] = acc
    for accept_g, accept_o in ((acc_world, acc), (None, None)):
        hg = g.raycast(rays, accept_g)
        ho = o.raycast(d[pre + "rays"], accept_o)
        assert np.array_equal(hg["body"], ho["body"])
        hit = ho["body"] >= 0
        assert hit.sum() >= min_hits
        assert np.array_equal(hg["collider"][hit], ho["collider"][hit])
        assert np.array_equal(hg["distance"][hit].view(np.uint32), ho["distance"][hit].view(np.uint32))
        assert np.array_equal(hg["pos"][hit].view(np.uint32), ho["pos"][hit].view(np.uint32))
    counts, hits = g.overlap(_queries(d, pre, scene), cap=256)
    total = 0
    for k, h in enumerate(hits):
        want = o.overlap(d[pre + "q_pos"][k], d[pre + "q_quat"][k], d[pre + "q_type"][k], d[pre + "q_params"][k],
                         d[pre + "q_mesh"][k], d[pre + "q_filter"][k])
        assert counts[k] == len(want)
        assert sorted((b, c) for b, c, _ in h) == sorted(want), k
        total += len(want)
    assert total >= min_hits
    counts, hits = g.overlap_mtd(_queries(d, pre, scene), cap=256)
    total = 0
    for k, h in enumerate(hits):
        want = make_golden.mtd_sorted(o.overlap_mtd(d[pre + "q_pos"][k], d[pre + "q_quat"][k], d[pre + "q_type"][k],
                                                    d[pre + "q_params"][k], d[pre + "q_mesh"][k]))
        got = make_golden.mtd_sorted([(b, c, n, m) for b, c, _, n, m in h])
        assert counts[k] == len(want)
        assert [(x[0], x[1]) for x in got] == [(x[0], x[1]) for x in want], k
        fg = np.asarray([list(x[2]) + [x[3]] for x in got], np.float32).reshape(-1, 4)
        fw = np.asarray([list(x[2]) + [x[3]] for x in want], np.float32).reshape(-1, 4)
        assert np.array_equal(fg.view(np.uint32), fw.view(np.uint32)), k
        total += len(want)
    assert total >= min_hits


@pytest.mark.parametrize("name", list(make_golden.query_scenes()))
def test_queries_match_oracle(gpu_lib, oracle_lib, name):
    d = np.load(os.path.join(HERE, "golden", "queries.npz"))
    s, frames = make_golden.query_scenes()[name]
    g, (o,) = _lockstep([s], frames)
    _check_scene(g, o, d, name + "__", 0, 0, g.counts()["bodies"])
    assert g.counts()["error"] == 0


def test_queries_in_a_batched_world(gpu_lib, oracle_lib):
    """Each scene of a batch answers its own queries as it does alone."""
    d = np.load(os.path.join(HERE, "golden", "queries.npz"))
    sc = make_golden.query_scenes()
    names = list(sc)
    frames = 5
    g, os_ = _lockstep([sc[n][0] for n in names], frames)
    for i, n in enumerate(names):
        # the fixture's rays and shapes aim at the bodies after its own frame counts: fewer hits here
        _check_scene(g, os_[i], d, n + "__", i, g.body_start[i], g.counts()["bodies"], min_hits=1)


def test_query_edge_cases(gpu_lib, oracle_lib):
    """A scene of one collider (no internal tree node), rays along an axis, a ray that
    starts inside a shape, a triangle-mesh query and a filter that no collider meets."""
    from physecs_gb300.api import World
    s = scenes.SceneData("one sphere")
    m, com, inertia = scenes.mass_sphere(0.5)
    s.add_bodies(pos=[[0, 1, 0]], quat=[scenes.IDENTITY_Q], flags=scenes.BODY_DYNAMIC, inv_mass=1.0 / m, com=com,
                 inv_inertia=np.linalg.inv(inertia).T.ravel(), col_type=scenes.SPHERE, col_params=[0.5, 0, 0, 0])
    g = World([s.finalize()])
    rays = np.array([[0, 0, 5, 0, 0, -1, 0, 10], [0, 0, 1, 0, 1, 0, 0, 10], [0, 3, 1, 0, 0, -1, 0, 10],
                     [0, 0.2, 5, 0, 0, -1, 0, 3]], np.float64)
    h = g.raycast(rays)
    assert list(h["body"]) == [0, 0, -1, -1]
    assert h["distance"][0] == np.float32(3.5) and h["distance"][1] == 0.0
    counts, hits = g.overlap([{"scene": 0, "pos": [0, 1, 0], "type": scenes.SPHERE, "params": [0.2]},
                              {"scene": 0, "pos": [0, 1, 0], "type": scenes.TRIANGLE_MESH, "params": [0, 0, 0]},
                              {"scene": 0, "pos": [0, 1, 0], "type": scenes.SPHERE, "params": [0.2], "filter": 4}])
    assert list(counts) == [1, 0, 0] and hits[0][0][:2] == (0, 0)
