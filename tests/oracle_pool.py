"""The CPU oracle over many scenes in spawned worker processes (test infrastructure).

A batched GPU world of thousands of scenes is checked scene by scene against the
oracle.  One oracle frame of the 4096-scene workload takes about ten seconds on one
core, so the scenes are split over worker processes, each owning the OracleScenes of
its share and rebuilding its scenes from their seeds.  Every frame the parent sends
each worker the GPU's results for its scenes (contact order, body state and, on the
frames that check them, pair sets, manifolds or creation bounds); the worker steps
its oracles in the GPU's contact order and sends back only the comparison results.

Workers are started with the "spawn" method, so they never inherit a CUDA context.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build_scene(spec):
    """spec = ("batch", index, config): one scene of the batched workload, with the
    workload's shared hull pool."""
    from physecs_gb300 import scenes
    kind, idx, config = spec
    assert kind == "batch"
    pool = _POOLS.get(config)
    if pool is None:
        pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(config, 1 << 19)), count=8)
        _POOLS[config] = pool
    return scenes.batch_scene(idx, config=config, pool=pool)


_POOLS = {}


def _worker(conn, specs):
    sys.path.insert(0, ROOT)
    from oracle.port_api import OracleScene
    from tests.parity import compare_contacts, pair_set, rel_state_diff
    ss = [_build_scene(sp) for sp in specs]
    os_ = [OracleScene(s) for s in ss]
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg is None:
            break
        out = {"state": 0.0, "order_error": 0, "pair_mismatch": [], "manifolds": 0.0, "bounds_mismatch": []}
        if msg["op"] == "bounds":
            for k, (s, o) in enumerate(zip(ss, os_)):
                gb = msg["bounds"][k]
                ids, ob = o.bounds()
                order = np.array([s.arrays["collider_start"][e] + c for e, c in ids])
                if not np.array_equal(gb[order].view(np.uint32), ob.view(np.uint32)):
                    out["bounds_mismatch"].append(k)
        else:
            for k, o in enumerate(os_):
                o.set_contact_order(msg["keys"][k])
                o.step()
                out["order_error"] += o.order_error()
                out["state"] = max(out["state"], rel_state_diff(msg["state"][k], o.state()))
                if msg.get("pairs") is not None:
                    if pair_set(msg["pairs"][k]) != pair_set(o.pairs()):
                        out["pair_mismatch"].append(k)
                if msg.get("contacts") is not None:
                    gk, gf = msg["contacts"][k]
                    _, of = o.contacts()
                    out["manifolds"] = max(out["manifolds"], compare_contacts(gk, gf, o.contact_keys(), of))
        conn.send(out)
    conn.close()


class OraclePool:
    """Oracle scenes for `specs` (one per GPU scene, in world order) spread over
    `procs` spawned processes in contiguous, body-balanced chunks."""

    def __init__(self, specs, weights, procs=None):
        procs = max(1, min(procs or (os.cpu_count() or 1), len(specs)))
        # contiguous chunks of about equal weight (bodies), so workers finish together
        cw = np.cumsum(np.asarray(weights, np.float64))
        cuts = np.searchsorted(cw, cw[-1] * np.arange(1, procs) / procs)
        bounds = [0] + sorted(set(int(c) + 1 for c in cuts if 0 < int(c) + 1 < len(specs))) + [len(specs)]
        self.chunks = [(bounds[i], bounds[i + 1]) for i in range(len(bounds) - 1)]
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for a, b in self.chunks:
            parent, child = ctx.Pipe()
            p = ctx.Process(target=_worker, args=(child, specs[a:b]), daemon=True)
            p.start()
            self.conns.append(parent)
            self.procs.append(p)
        for c in self.conns:
            assert c.recv() == "ready"

    def _round(self, msgs):
        for c, m in zip(self.conns, msgs):
            c.send(m)
        res = [c.recv() for c in self.conns]
        out = {"state": max(r["state"] for r in res), "order_error": sum(r["order_error"] for r in res),
               "manifolds": max(r["manifolds"] for r in res), "pair_mismatch": [], "bounds_mismatch": []}
        for (a, _), r in zip(self.chunks, res):
            out["pair_mismatch"] += [a + k for k in r["pair_mismatch"]]
            out["bounds_mismatch"] += [a + k for k in r["bounds_mismatch"]]
        return out

    def check_bounds(self, per_scene_bounds):
        return self._round([{"op": "bounds", "bounds": per_scene_bounds[a:b]} for a, b in self.chunks])

    def step(self, keys, states, pairs=None, contacts=None):
        """keys, states (and pairs, contacts when given): per-scene lists in world order."""
        msgs = []
        for a, b in self.chunks:
            msgs.append({"op": "step", "keys": keys[a:b], "state": states[a:b],
                         "pairs": None if pairs is None else pairs[a:b],
                         "contacts": None if contacts is None else contacts[a:b]})
        return self._round(msgs)

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except Exception:
                pass
        for p in self.procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
        self.conns, self.procs = [], []
