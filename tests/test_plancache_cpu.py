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


class FakeVoxelLib:
    """Stand-in for the native library's set-atoms/shells calls: records
    the atom counts and fails on request."""

    def __init__(self):
        self.counts, self.fail = [], False

    def gw_voxel_set_atoms(self, handle, xyz, f, n, on_device):
        self.counts.append(n)
        return 1 if self.fail else 0

    def gw_voxel_set_shells(self, *args):
        return 0


def test_graph_flag_follows_atom_count_and_shells(monkeypatch):
    """The library drops a plan's recorded graph when the atom count or
    the shells change; the host flag that says a graph is recorded follows."""
    import numpy as np
    from giwaxsim_gb300 import _native as N
    from giwaxsim_gb300.forward import VoxelPlan
    fake = FakeVoxelLib()
    monkeypatch.setattr(N, "lib", lambda: fake)
    monkeypatch.setattr(N, "last_error", lambda: "fake failure")
    plan = VoxelPlan.__new__(VoxelPlan)
    plan.handle, plan.graph_captured, plan._atoms_n = object(), False, None
    x4, x5 = np.zeros((4, 3)), np.zeros((5, 3))
    f4, f5 = np.zeros(8, np.float32), np.zeros(10, np.float32)
    plan.set_atoms(x4, f4)
    plan.graph_captured = True           # as capture_graph() leaves it
    plan.set_atoms(x4, f4)               # same count: the graph stays
    assert plan.graph_captured
    plan.set_atoms(x5, f5)               # new count: the library drops it
    assert not plan.graph_captured
    plan.graph_captured = True
    fake.fail = True                     # a failed upload leaves no count
    try:
        plan.set_atoms(x4, f4)
    except N.GwError:
        pass
    assert not plan.graph_captured and plan._atoms_n is None
    fake.fail = False
    plan.set_atoms(x4, f4)
    plan.graph_captured = True
    plan.set_shells(None, None, None, None, None)
    assert not plan.graph_captured
    assert fake.counts == [4, 4, 5, 4, 4]


def test_default_context_is_per_thread(monkeypatch):
    """default_context() gives each thread its own context (own stream and
    error word) and the same one on every call within a thread."""
    import threading
    from giwaxsim_gb300 import _native as N

    class FakeContext:
        def __init__(self, device=0):
            self.device = device
    monkeypatch.setattr(N, "Context", FakeContext)
    monkeypatch.setattr(N, "_thread_contexts", threading.local())
    main = N.default_context()
    assert N.default_context() is main and N.default_context(1) is not main
    got = []

    def worker():
        got.append((N.default_context(), N.default_context()))
    ts = [threading.Thread(target=worker) for _ in range(3)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert all(a is b for a, b in got)
    ids = {id(a) for a, _ in got}
    assert len(ids) == 3 and id(main) not in ids


def test_detector_model_keeps_one_context(monkeypatch):
    """A DetectorModel made without ctx takes the constructing thread's
    context and hands the same one to its detector plan (its forward's
    voxel plans use self.ctx too), so a forward called from another thread
    stays on one stream."""
    import threading
    from giwaxsim_gb300 import _native as N
    from giwaxsim_gb300 import autograd as A

    class FakeContext:
        def __init__(self, device=0):
            self.device = device
    got = {}

    class FakeDetectorPlan:
        def __init__(self, *args, ctx=None, **kw):
            got["det_ctx"] = ctx
    monkeypatch.setattr(N, "Context", FakeContext)
    monkeypatch.setattr(N, "_thread_contexts", threading.local())
    monkeypatch.setattr(A, "DetectorPlan", FakeDetectorPlan)
    m = A.DetectorModel(["C"] * 4, 10000.0, 0.5, 0.15, 1.5, 16)
    assert m.ctx is N.default_context() and got["det_ctx"] is m.ctx
    seen = []
    t = threading.Thread(target=lambda: seen.append(N.default_context()))
    t.start()
    t.join()
    assert seen[0] is not m.ctx


def test_host_pool_recycles_pinned_buffers(monkeypatch):
    """A kept buffer is page-locked once, handed out again once its result
    is dropped, and unlocked by clear() (the pool keeps addresses, not
    references, of what it locked)."""
    import numpy as np
    from giwaxsim_gb300 import _native as N
    from giwaxsim_gb300.forward import HostPool

    class FakePin:
        def __init__(self):
            self.pinned, self.unpinned = [], []

        def gw_host_pin(self, ptr, n):
            self.pinned.append(ptr.value)
            return 0

        def gw_host_unpin(self, ptr):
            self.unpinned.append(ptr.value)
            return 0

    fake = FakePin()
    monkeypatch.setattr(N, "lib", lambda: fake)
    pool = HostPool(min_bytes=1 << 20, per_shape=1)
    a = pool.empty((256, 1024))
    ptr = a.ctypes.data
    del a
    b = pool.empty((256, 1024))
    assert b.ctypes.data == ptr and fake.pinned == [ptr]
    c = pool.empty((256, 1024))          # b still held: a fresh, unkept one
    assert c.ctypes.data != ptr and fake.pinned == [ptr]
    small = pool.empty((4, 4))           # below min_bytes: never locked
    assert small.shape == (4, 4) and fake.pinned == [ptr]
    pool.clear()
    assert fake.unpinned == [ptr] and pool._pinned == []
    b[:] = 1.0
    assert b.sum() == 256 * 1024
