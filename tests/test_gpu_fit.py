"""Separate-structure voxel plans and the slab-size fit loop."""
import numpy as np
import pytest

from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.fit import SlabFit

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_separate_structures_match_single_plans():
    """One batched plan with a separate I(q) per structure equals one plan
    per structure."""
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.linspace(0.0, 180.0, 12, endpoint=False)
    rng = np.random.default_rng(3)
    items = []
    for size in ((10.0, 12.0, 9.0), (14.0, 11.0, 13.0), (9.0, 9.0, 16.0)):
        xyz, _ = W.graphite_slab(size, rng, disp_sigma=0.05)
        items.append((xyz, np.full(len(xyz), 6.0 + 0j), None))
    plan = F.VoxelPlan(geom, items, phis=phis, smooth=1.5, average="separate")
    plan.set_atoms()
    plan.execute()
    iq = plan.iq()
    assert iq.shape == (3,) + (plan.Qc,) * 3
    for k, it in enumerate(items):
        p1 = F.VoxelPlan(geom, [it], phis=phis, smooth=1.5)
        p1.set_atoms()
        p1.execute()
        assert rel_l2(iq[k], p1.iq()) <= 1e-6
        p1.close()
    plan.close()


def _graphite_problem(true_size):
    cell = W.GRAPHITE_BASIS @ W.GRAPHITE_CELL
    cellp = (2.46, 2.46, 6.70, 90.0, 90.0, 120.0)
    kw = dict(r_voxel_size=0.4, q_voxel_size=0.08, max_q=2.0, energy=10000.0,
              num_pixels=64, phis=np.linspace(0, 180, 24, endpoint=False),
              psis=np.linspace(0, 180, 10))
    # the experiment: the positive quadrant of the image of a slab of the
    # true size (what simulate_GIWAXS saves)
    probe = SlabFit(cell, ["C"] * 4, cellp, exp_img=np.ones((2, 2)),
                    exp_qxy=np.array([0.0, 2.0]), exp_qz=np.array([0.0, 2.0]),
                    exp_mask=np.zeros((2, 2)), **kw)
    img = probe.images([true_size])[0]
    h, v = probe.det.det_h, probe.det.det_v
    probe.close()
    kh, kv = np.where(h >= 0)[0], np.where(v >= 0)[0]
    exp = img[np.ix_(kv, kh)]
    fit = SlabFit(cell, ["C"] * 4, cellp, exp_img=exp, exp_qxy=h[kh],
                  exp_qz=v[kv], exp_mask=np.zeros_like(exp), **kw)
    return fit


def test_fit_misfit_zero_at_the_true_size_and_grid_improves():
    true = np.array([30.0, 28.0, 27.0])
    fit = _graphite_problem(true)
    (s, o, m0), (s1, o1, m1) = fit.misfits([true, true * np.array([1.2, 1.0, 1.0])])
    # the experiment is the simulation itself on the same grid: scale 1,
    # offset 0, misfit at the rounding level of the moment sums
    t, _ = fit.cmp.target()
    assert abs(s - 1.0) < 1e-6 and abs(o) < 1e-6 * np.abs(t).max()
    assert m0 < 1e-9 * m1
    init = true * np.array([1.15, 1.0, 1.0])
    res = fit.fit(init, vary=(True, False, False), method="grid",
                  grid_points=5, rounds=3, step=0.2)
    m_init = fit.misfits([init])[0][2]
    assert res["misfit"] <= m_init
    assert abs(res["size"][0] - true[0]) < 0.1 * true[0]
    res2 = fit.fit(init, vary=(True, False, False), method="nelder-mead",
                   max_evals=8)
    assert res2["evaluations"] <= 8 and res2["misfit"] <= m_init
    fit.close()
