"""psx_world_read_bodies_noalloc against psx_world_read_bodies, through the C ABI.

Collected last on purpose: it must also pass after every other test has run in
the same process (the fixed device array then holds another world's data)."""
import ctypes as C

import numpy as np
import pytest

from physecs_gb300 import scenes

pytestmark = pytest.mark.gpu

# Both calls return the same float32 values copied from the same device state;
# the tolerance is exact equality.
TOL = 0.0


def _empty(n):
    return dict(pos=np.full((n, 3), np.nan, np.float32), quat=np.full((n, 4), np.nan, np.float32),
                vel=np.full((n, 3), np.nan, np.float32), ang_vel=np.full((n, 3), np.nan, np.float32))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _read(lib, fn, w, keys=("pos", "quat", "vel", "ang_vel")):
    st = _empty(w.n_bodies)
    args = [_p(st[k]) if k in keys else None for k in ("pos", "quat", "vel", "ang_vel")]
    status = getattr(lib, fn)(w.h, *args)
    assert status == 0, lib.psx_last_error_string()
    return st


def _assert_same(a, b, keys=("pos", "quat", "vel", "ang_vel")):
    for k in keys:
        assert np.isfinite(a[k]).all(), k
        d = np.abs(a[k].astype(np.float64) - b[k].astype(np.float64)).max()
        assert d <= TOL, (k, d)


def _world_with_kinematic():
    """Three uneven scenes; one body of the second scene made kinematic."""
    ss = [scenes.batch_scene(41, n_bodies=50), scenes.batch_scene(42, n_bodies=90, chain_prob=1.0),
          scenes.batch_scene(43, n_bodies=30)]
    f = ss[1].arrays["flags"]
    k = int(np.nonzero(f & scenes.BODY_DYNAMIC)[0][3])
    f[k] |= scenes.BODY_KINEMATIC
    return ss


def test_noalloc_read_matches_read_on_consecutive_calls():
    from physecs_gb300.api import World, load
    lib = load()
    w = World(_world_with_kinematic())
    for call in range(2):
        w.step()
        a = _read(lib, "psx_world_read_bodies", w)
        b = _read(lib, "psx_world_read_bodies_noalloc", w)
        _assert_same(a, b)
        # static bodies report zero velocity, not stale scratch contents
        static = np.array([not (fl & scenes.BODY_DYNAMIC) for s in w.scenes for fl in s.arrays["flags"]])
        assert static.any()
        assert (b["vel"][static] == 0).all() and (b["ang_vel"][static] == 0).all()
    # a subset of outputs (NULL for the others)
    w.step()
    a = _read(lib, "psx_world_read_bodies", w)
    b = _read(lib, "psx_world_read_bodies_noalloc", w, keys=("quat", "ang_vel"))
    _assert_same(a, b, keys=("quat", "ang_vel"))
    assert np.isnan(b["pos"]).all() and np.isnan(b["vel"]).all()


def test_noalloc_read_after_a_larger_world():
    """The array keeps the previous call's contents: a smaller world read after a larger
    one must see only its own bodies."""
    from physecs_gb300.api import World, load
    lib = load()
    big = World([scenes.batch_scene(50 + i, n_bodies=400) for i in range(4)])
    small = World(scenes.batch_scene(60, n_bodies=20))
    big.step()
    small.step()
    for _ in range(2):
        _read(lib, "psx_world_read_bodies_noalloc", big)
        b = _read(lib, "psx_world_read_bodies_noalloc", small)
        _assert_same(_read(lib, "psx_world_read_bodies", small), b)
        small.step()
        big.step()


def test_noalloc_read_rejects_worlds_over_the_limit():
    from physecs_gb300.api import World, load
    lib = load()
    s = scenes.pyramid(rows=12)              # 78 boxes + ground
    n = len(s.arrays["pos"])
    w = World([s] * (65536 // n + 1))
    assert w.n_bodies > 65536
    st = _empty(w.n_bodies)
    status = lib.psx_world_read_bodies_noalloc(w.h, _p(st["pos"]), None, None, None)
    assert status == 3  # PSX_ERR_CAPACITY
    msg = lib.psx_last_error_string().decode()
    assert "65536" in msg
    assert np.isnan(st["pos"]).all()
