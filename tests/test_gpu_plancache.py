"""The drop-in voxel call keeps its plan for the next call with the same
plan inputs: repeated and interleaved calls give the results of a plan
made for each call."""
import numpy as np
import pytest

from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import comparison as C

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def fresh_iq(xyz, el, r, dq, max_q, energy, phis, smooth):
    geom = F.VoxelGeometry(r, dq, max_q)
    fv = F.element_f_values(el, energy)
    p = F.VoxelPlan(geom, [(xyz, fv, None)], phis=phis, smooth=smooth)
    try:
        p.set_atoms()
        p.execute()
        return p.iq().copy()
    finally:
        p.close()


def test_repeated_and_interleaved_calls():
    rng = np.random.default_rng(11)
    a, _ = W.graphite_slab((10.0, 12.0, 9.0), rng, disp_sigma=0.05)
    b, _ = W.graphite_slab((13.0, 9.0, 11.0), rng, disp_sigma=0.05)
    # same extents and f sum as a (the plan's inputs), other positions:
    # pulled towards the centre, the extreme atoms of every axis kept
    c = 0.5 * (a.max(0) + a.min(0))
    a2 = c + 0.97 * (a - c)
    for ax in range(3):
        for i in (np.argmin(a[:, ax]), np.argmax(a[:, ax])):
            a2[i] = a[i]
    el_a, el_b = ["C"] * len(a), ["C"] * len(b)
    kw = dict(r_voxel_size=0.5, q_voxel_size=0.15, max_q=1.5, energy=10000.0)
    phis = np.linspace(0.0, 180.0, 12, endpoint=False)
    C.PLAN_CACHE.clear()
    ref = {k: fresh_iq(x, e, 0.5, 0.15, 1.5, 10000.0, phis, 1.0)
           for k, (x, e) in {"a": (a, el_a), "b": (b, el_b), "a2": (a2, el_a)}.items()}
    seq = ["a", "a", "b", "a", "a2", "a", "b", "b"]
    inputs = {"a": (a, el_a), "b": (b, el_b), "a2": (a2, el_a)}
    handles, graphs = [], []
    for k in seq:
        x, e = inputs[k]
        iq, qx, qy, qz = C.voxelgridmaker_fitting(x, e, smooth=1.0, phis=phis, **kw)
        assert rel_l2(iq, ref[k]) <= 1e-9, k
        assert len(C.PLAN_CACHE._plans) == 1
        kept = next(iter(C.PLAN_CACHE._plans.values()))
        handles.append(kept.handle.value)
        graphs.append(kept.graph_captured)
    # the second call of a reused the first call's plan, and a2 (other
    # atoms, equal plan inputs) the plan of the call before it
    assert handles[1] == handles[0]
    assert handles[4] == handles[3]
    # a reused plan runs as a recorded graph: a2 and the a after it were
    # replays of the graph recorded with other atoms in the buffers
    assert graphs == [False, True, False, False, True, True, False, True]
    assert rel_l2(ref["a2"], ref["a"]) > 1e-3
    C.PLAN_CACHE.clear()
    assert len(C.PLAN_CACHE._plans) == 0


def test_failed_call_drops_its_plan():
    rng = np.random.default_rng(12)
    a, _ = W.graphite_slab((8.0, 8.0, 8.0), rng, disp_sigma=0.05)
    kw = dict(r_voxel_size=0.5, q_voxel_size=0.15, max_q=1.5, energy=10000.0)
    C.PLAN_CACHE.clear()
    C.voxelgridmaker_fitting(a, ["C"] * len(a), phis=[0.0, 90.0], **kw)
    assert len(C.PLAN_CACHE._plans) == 1
    with pytest.raises(Exception):
        # an unknown element fails before any plan work
        C.voxelgridmaker_fitting(a, ["Xx"] * len(a), phis=[0.0, 90.0], **kw)
    assert len(C.PLAN_CACHE._plans) == 1
    C.PLAN_CACHE.clear()


def test_result_copy_into_resident_buffer_fills_every_line():
    """A resident host destination (copied in one call): prefilled with
    NaN, every voxel is overwritten, lines without a binned pixel with
    zeros, on repeated calls."""
    rng = np.random.default_rng(13)
    xyz, _ = W.graphite_slab((12.0, 10.0, 9.0), rng, disp_sigma=0.05)
    geom = F.VoxelGeometry(0.5, 0.1, 1.5)
    fv = F.element_f_values(["C"] * len(xyz), 10000.0)
    plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=np.linspace(0, 170, 8),
                       smooth=1.0)
    try:
        plan.set_atoms()
        plan.execute()
        ref32 = plan.iq32()   # copied by the copy engine, one float32 per voxel
        counts = plan.counts()
        empty_lines = (counts.reshape(plan.Qc * plan.Qc, plan.Qc) == 0).all(1)
        assert 0.05 < empty_lines.mean() < 0.95   # both kinds of line exist
        out = np.full((plan.Qc,) * 3, np.nan)
        for _ in range(2):
            out[:] = np.nan
            plan.iq(out=out)
            assert not np.isnan(out).any()
            # the float32 result (float32 arithmetic) is within 2 ulps of
            # the float64 one rounded, and zero where it is
            r32 = out.astype(np.float32)
            assert np.array_equal(r32 == 0, ref32 == 0)
            ulps = np.abs(r32.view(np.int32).astype(np.int64)
                          - ref32.view(np.int32).astype(np.int64))
            assert ulps.max() <= 2
        assert np.all(out.reshape(-1, plan.Qc)[empty_lines] == 0)
        assert np.any(out.reshape(-1, plan.Qc)[~empty_lines] != 0)
    finally:
        plan.close()


def test_host_pool_pins_kept_buffers():
    """Kept result buffers are page-locked once and released by clear();
    a buffer handed out again is the same memory."""
    pool = F.HostPool(min_bytes=1 << 20, per_shape=1)
    a = pool.empty((256, 1024))
    assert len(pool._pinned) == 1
    ptr = a.ctypes.data
    del a
    b = pool.empty((256, 1024))          # recycled: no second page lock
    assert b.ctypes.data == ptr and len(pool._pinned) == 1
    c = pool.empty((256, 1024))          # b still held: a fresh, unkept one
    assert c.ctypes.data != ptr and len(pool._pinned) == 1
    pool.clear()
    assert pool._pinned == []
    b[:] = 1.0                           # still ordinary memory
    assert b.sum() == 256 * 1024
