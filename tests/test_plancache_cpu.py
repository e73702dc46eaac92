"""PlanCache bookkeeping with stand-in plans (no device)."""
from giwaxsim_gb300.forward import PlanCache


class FakePlan:
    def __init__(self, key):
        self._key, self.handle, self.closed = key, object(), False

    def key(self):
        return self._key

    def close(self):
        self.closed, self.handle = True, None


def test_keep_evict_and_failures():
    c = PlanCache(size=2)
    p1, p2, p3 = FakePlan("a"), FakePlan("b"), FakePlan("c")
    for p in (p1, p2):
        c.give_back(p)
    assert list(c._plans) == ["a", "b"] and not p1.closed
    c.give_back(p3)                      # over capacity: least recent goes
    assert list(c._plans) == ["b", "c"] and p1.closed
    p4 = FakePlan("b")
    c.give_back(p4)                      # same key again: the older is destroyed
    assert c._plans["b"] is p4 and p2.closed
    p5 = FakePlan("d")
    c.give_back(p5, ok=False)            # a failed call's plan is not kept
    assert p5.closed and "d" not in c._plans
    c.clear()
    assert not c._plans and p3.closed and p4.closed


def test_size_zero_keeps_nothing():
    c = PlanCache(size=0)
    p = FakePlan("a")
    c.give_back(p)
    assert p.closed and not c._plans
