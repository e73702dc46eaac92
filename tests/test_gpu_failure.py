"""Failure paths of the library, exercised without faulting the GPU.

The reference's failure surface is Python exceptions: geometry errors
(tools/comparison.py:705-717) and weight asserts (:826-832).  The library
adds two of its own, both turned into Python exceptions (GwError with the
gw_status) that leave the context usable:
  * a device allocation that fails (injected on the host with the
    gw_set_alloc_fault hook) -> GW_ERR_OOM;
  * the column kernel's bounded wait for its TMA tile load running out (the
    limit set to 0 polls with gw_voxel_set_wait_limit) -> GW_ERR_TIMEOUT.
"""
import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import comparison
from oracle import giwaxs_oracle as O

pytestmark = pytest.mark.gpu


def _case(seed=0, size=(12.0, 11.0, 13.0)):
    rng = np.random.default_rng(seed)
    xyz, _ = W.graphite_slab(size, rng, disp_sigma=0.05)
    return xyz, np.array(["C"] * len(xyz))


def _plan(ctx, xyz, phis, r=0.5, dq=0.15, mq=1.5):
    geom = F.VoxelGeometry(r, dq, mq)
    fv = F.element_f_values(["C"] * len(xyz), 10000.0)
    plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=phis, fill_bkg=True,
                       smooth=1, ctx=ctx)
    plan.set_atoms()
    return plan


def test_injected_allocation_failure_raises_and_context_recovers():
    ctx = N.Context(0)
    xyz, el = _case()
    phis = np.array([0.0, 33.0, 90.0, 151.0])
    plan = _plan(ctx, xyz, phis)
    plan.execute()
    ctx.synchronize()
    ref = plan.iq().copy()
    N.set_alloc_fault(0)
    try:
        with pytest.raises(N.GwError) as e:
            _plan(ctx, xyz, phis, dq=0.14)       # a new plan must allocate
        assert e.value.status == N.GW_ERR_OOM
        # the drop-in API raises the same way (a shape it has no plan for)
        with pytest.raises(N.GwError) as e:
            comparison.voxelgridmaker_fitting(xyz, el, 0.5, 0.13, 1.5, 10000.0,
                                              fill_bkg=True, smooth=1,
                                              phis=phis, ctx=ctx)
        assert e.value.status == N.GW_ERR_OOM
    finally:
        N.set_alloc_fault(-1)
    # the context and the plan made before still work, and new plans again
    plan.execute()
    ctx.synchronize()
    assert np.allclose(plan.iq(), ref, rtol=1e-12, atol=0)
    iq, _, _, _ = comparison.voxelgridmaker_fitting(
        xyz, el, 0.5, 0.13, 1.5, 10000.0, fill_bkg=True, smooth=1, phis=phis,
        ctx=ctx)
    want = O.voxelgrid([(xyz, np.full(len(xyz), 6.0 + 0j))], 0.5, 0.13, 1.5,
                       phis, True, 1)["iq"]
    assert np.linalg.norm(iq - want) / np.linalg.norm(want) <= 1e-5
    plan.close()
    ctx.close()


def test_tile_wait_timeout_reports_and_context_recovers():
    ctx = N.Context(0)
    xyz, _ = _case(1)
    phis = np.array([0.0, 21.0, 60.0, 97.0, 140.0])
    plan = _plan(ctx, xyz, phis)
    assert plan.info()["col_tma"] == 1, "this plan's column kernel must use TMA"
    plan.execute()
    ctx.synchronize()
    ref = plan.iq().copy()
    plan.set_wait_limit(0)               # every tile wait runs out at once
    plan.execute()
    with pytest.raises(N.GwError) as e:
        ctx.synchronize()
    assert e.value.status == N.GW_ERR_TIMEOUT
    assert "bounded wait" in str(e.value)
    plan.set_wait_limit(1 << 22)
    plan.execute()
    ctx.synchronize()                    # no error left behind
    assert np.allclose(plan.iq(), ref, rtol=1e-12, atol=0)
    # a captured graph keeps the limit it was captured with until it is set
    plan.capture_graph()
    plan.set_wait_limit(0)
    assert not plan.graph_captured
    plan.execute()
    with pytest.raises(N.GwError):
        ctx.synchronize()
    plan.set_wait_limit(1 << 22)
    plan.capture_graph()
    plan.execute()
    ctx.synchronize()
    assert np.allclose(plan.iq(), ref, rtol=1e-12, atol=0)
    plan.close()
    ctx.close()
