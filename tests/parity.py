"""Shared comparison helpers for the parity tests (GPU path vs CPU oracle)."""
from __future__ import annotations

import numpy as np


def gpu_keys(ids, meta):
    """Manifold keys {entity0, collider0, entity1, collider1, triangleIndex} of GPU contacts."""
    return np.concatenate([ids[:, 4:8], meta[:, 1:2]], axis=1).astype(np.int32)


def pair_set(rows):
    return set(map(tuple, np.asarray(rows).tolist()))


def contact_table(keys, f):
    """dict key -> 56-float contact row."""
    return {tuple(k): row for k, row in zip(np.asarray(keys).tolist(), f)}


def compare_contacts(gk, gf, ok, of, atol=1e-5):
    """Max abs difference of matched manifold data (normal, friction, r0, r1, targetVelocity)."""
    g = contact_table(gk, gf)
    o = contact_table(ok, of)
    assert set(g) == set(o), "manifold key sets differ: %d gpu vs %d oracle, %d common" % (len(g), len(o), len(set(g) & set(o)))
    worst = 0.0
    cols = list(range(0, 4)) + [8 + 12 * k + j for k in range(4) for j in range(7)]
    for k in g:
        x, y = g[k][cols].astype(np.float64), o[k][cols].astype(np.float64)
        if not np.array_equal(np.isnan(x), np.isnan(y)):
            return float("inf")
        ok = ~np.isnan(x)
        if ok.any():
            worst = max(worst, float(np.abs(x[ok] - y[ok]).max()))
    return worst


def state_diff(a, b, sl=slice(None)):
    out = 0.0
    for k in ("pos", "quat", "vel", "ang_vel"):
        d = np.abs(a[k][sl].astype(np.float64) - b[k][sl].astype(np.float64))
        if np.isnan(d).any():
            return float("inf")
        out = max(out, float(d.max()))
    return out


def rel_state_diff(a, b, sl=slice(None)):
    """max |a-b| / max(1, |b|) over all state components.  A NaN counts as equal only
    to a NaN in the same place; any other NaN makes the difference infinite."""
    worst = 0.0
    for k in ("pos", "quat", "vel", "ang_vel"):
        x, y = a[k][sl].astype(np.float64), b[k][sl].astype(np.float64)
        nx, ny = np.isnan(x), np.isnan(y)
        if not np.array_equal(nx, ny):
            return float("inf")
        ok = ~nx
        if ok.any():
            worst = max(worst, float((np.abs(x[ok] - y[ok]) / np.maximum(1.0, np.abs(y[ok]))).max()))
    return worst
