"""World.dispatch_trigger_events on canned events (no device): listeners of each scene in
registration order, every entering pair calling every enter listener and every exiting
pair every exit listener, in the delivered order; removal; lost events raised only after
the dispatch (src/Physecs.cpp:537-552, 772-786)."""
import numpy as np
import pytest

from physecs_gb300.api import PsxError, World


class _Log:
    def __init__(self, log, tag):
        self.log, self.tag = log, tag

    def on_trigger_enter(self, e0, c0, e1, c1):
        self.log.append((self.tag, "enter", e0, c0, e1, c1))

    def on_trigger_exit(self, e0, c0, e1, c1):
        self.log.append((self.tag, "exit", e0, c0, e1, c1))


def _world(events, lost=0):
    w = World.__new__(World)          # no library call: trigger_events is replaced below
    w.trigger_events = lambda cap=4096: (np.asarray(events, np.int64).reshape(-1, 9), lost)
    return w


# (frame, kind, scene, body0, collider0, body1, collider1, entity0, entity1)
EVENTS = [(0, 0, 0, 1, 0, 2, 0, 11, 12), (0, 0, 1, 3, 1, 4, 0, 13, 14), (0, 1, 0, 5, 0, 6, 2, 15, 16),
          (1, 0, 0, 7, 0, 8, 0, 17, 18)]


def test_dispatch_order_and_scenes():
    log = []
    w = _world(EVENTS)
    a, b, c = _Log(log, "a"), _Log(log, "b"), _Log(log, "c")
    w.add_on_trigger_enter_callback(a)
    w.add_on_trigger_enter_callback(b)
    w.add_on_trigger_exit_callback(a)
    w.add_on_trigger_enter_callback(c, scene=1)
    w.dispatch_trigger_events()
    assert log == [("a", "enter", 11, 0, 12, 0), ("b", "enter", 11, 0, 12, 0), ("c", "enter", 13, 1, 14, 0),
                   ("a", "exit", 15, 0, 16, 2), ("a", "enter", 17, 0, 18, 0), ("b", "enter", 17, 0, 18, 0)]


def test_remove_and_lost_events():
    log = []
    w = _world(EVENTS, lost=3)
    a = _Log(log, "a")
    w.add_on_trigger_enter_callback(a)
    w.remove_on_trigger_enter_callback(a)
    with pytest.raises(ValueError):
        w.remove_on_trigger_enter_callback(a)
    b = _Log(log, "b")
    w.add_on_trigger_exit_callback(b)
    with pytest.raises(PsxError):
        w.dispatch_trigger_events()
    assert log == [("b", "exit", 15, 0, 16, 2)]    # delivered before the loss is reported
