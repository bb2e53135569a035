"""A bounded device wait that runs out returns PSX_ERR_TIMEOUT and leaves the GPU usable.

A scene above the block limit, solved by the whole grid, waits at a grid barrier
between colour steps.  With the wait limited to one poll, a block that reaches a
barrier before the others gives up at once: it records the timeout, every block
leaves the solver, and the host reads PSX_ERR_TIMEOUT.  No fault and no hang is
involved: each wait ends after its bounded number of polls.  A world created
afterwards steps in lockstep with the oracle, so the context is intact.
"""
import time

import pytest

from physecs_gb300 import scenes
from tests.parity import gpu_keys, rel_state_diff

pytestmark = pytest.mark.gpu


def _grid_world(s):
    from physecs_gb300.api import World
    g = World([s], block_scene_max_dyn=64, launch={"large_scene_solver": 2})
    assert g.launch_config()["large_scene_solver"] == 2
    return g


def test_grid_wait_that_runs_out_reports_timeout(gpu_lib, oracle_lib):
    from oracle.port_api import OracleScene
    from physecs_gb300.api import PsxError
    s = scenes.batch_scene(31, n_bodies=300)
    g = _grid_world(s)
    g.set_wait_limit(1)
    t = time.perf_counter()
    g.step()
    with pytest.raises(PsxError, match="TIMEOUT"):
        g.synchronize()
    assert time.perf_counter() - t < 5.0
    g.close()
    # the default limit: a fresh world on the same device runs and matches the oracle
    g = _grid_world(s)
    o = OracleScene(s)
    for f in range(5):
        g.step()
        g.synchronize()
        ids, _, meta = g.contacts()
        o.set_contact_order(gpu_keys(ids, meta))
        o.step()
        assert o.order_error() == 0
        assert rel_state_diff(g.read_bodies(), o.state()) <= 1e-5, f
    assert g.counts()["error"] == 0
    # and the limit set back to the default on a world that stepped before
    g.set_wait_limit(0)
    g.step(frames=2)
    g.synchronize()
    g.close()
