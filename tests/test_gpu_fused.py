"""The fused chirp-z kernels (gw_czt2.cuh: one radix-R1 pass, a middle pass
holding the spectrum product in registers, one inverse radix-R1 pass)
against the Stockham kernels and the float64 oracle, over every option the
voxel stage has: fill/smoothing, the bilinear deposit, Kahan float32
accumulation, several structures with their own z windows, separate
per-structure grids, multi-q shells, graph replay, every block shape, and
both the half-length (window and band within M/2, pruned passes) and the
full-length forms.  Counts bit-exact; intensities by normwise relative L2
<= 1e-5 against the oracle and between the two kernel families."""
import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from oracle import giwaxs_oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(
        np.linalg.norm(np.asarray(b)), 1e-300)


def run(geom, structures, phis, fill, smooth, **kw):
    plan = F.VoxelPlan(geom, structures, phis=phis, fill_bkg=fill,
                       smooth=smooth, **kw)
    plan.set_atoms()
    plan.execute()
    out = dict(iq=plan.iq(), counts=plan.counts(), info=plan.info())
    plan.close()
    return out


def graphite(seed, size):
    rng = np.random.default_rng(seed)
    xyz, _ = W.graphite_slab(size, rng, disp_sigma=0.05)
    return xyz, np.full(len(xyz), 6.0 + 0j)


@pytest.mark.parametrize("m", [1024, 1280])
@pytest.mark.parametrize("fill,smooth", [(False, 0), (True, 1.5)])
def test_fused_half_vs_stockham_and_oracle(m, fill, smooth):
    xyz, fv = graphite(11, (12.0, 11.0, 13.0))
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.array([0.0, 17.0, 45.0, 90.0, 133.5])
    ref = O.voxelgrid([(xyz, fv)], 0.5, 0.15, 1.5, phis, fill, smooth)
    st = run(geom, [(xyz, fv, None)], phis, fill, smooth, fft_y=m, fft_z=m,
             transform="stockham")
    assert (st["info"]["fused_y"], st["info"]["fused_z"]) == (0, 0)
    for v in range(N.fused_variant_count()):
        fu = run(geom, [(xyz, fv, None)], phis, fill, smooth, fft_y=m, fft_z=m,
                 transform="fused", block_variant=v)
        assert (fu["info"]["fused_y"], fu["info"]["fused_z"]) == (1, 1)
        assert np.array_equal(fu["counts"], ref["count"])
        assert rel_l2(fu["iq"], ref["iq"]) <= RTOL, v
        assert rel_l2(fu["iq"], st["iq"]) <= RTOL, v


def test_fused_full_length_vs_oracle():
    """A window longer than M/2 along both axes (a 10 x 170 x 140 A Si
    slab at r = 0.25 A, dq = 0.02 1/A: Ly + Nc - 1 <= 1280 with Ly > 640,
    Lz + Nr - 1 <= 1024 with Lz > 512): the unpruned passes."""
    rng = np.random.default_rng(5)
    xyz, _ = W.silicon_slab((10.0, 170.0, 140.0), rng, disp_sigma=0.05)
    fv = np.full(len(xyz), 14.0 + 0j)
    geom = F.VoxelGeometry(0.25, 0.02, 4.0)
    phis = np.array([0.0, 3.0, 45.0, 120.0])
    fu = run(geom, [(xyz, fv, None)], phis, True, 2, transform="fused")
    info = fu["info"]
    assert (info["My"], info["Mz"]) == (1280, 1024), info
    assert info["Ly"] > 640 and info["Lz"] > 512, info
    ref = O.voxelgrid([(xyz, fv)], 0.25, 0.02, 4.0, phis, True, 2)
    assert np.array_equal(fu["counts"], ref["count"])
    assert rel_l2(fu["iq"], ref["iq"]) <= RTOL


@pytest.mark.parametrize("opt", ["bilinear", "kahan32", "structs", "separate",
                                 "graph", "shells"])
def test_fused_options_vs_stockham(opt):
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.array([0.0, 23.0, 61.0, 90.0, 144.0])
    xyz, fv = graphite(12, (12.0, 11.0, 13.0))
    structures = [(xyz, fv, None)]
    kw = {}
    if opt == "bilinear":
        kw["deposit"] = "bilinear"
    elif opt == "kahan32":
        kw["accum"] = "kahan32"
    elif opt in ("structs", "separate"):
        x2, f2 = graphite(13, (9.0, 14.0, 7.0))
        x3, f3 = graphite(14, (13.0, 8.0, 10.0))
        structures += [(x2, f2, None), (x3, f3, None)]
        if opt == "separate":
            kw["average"] = "separate"
    outs = {}
    for tr in ("fused", "stockham"):
        # shells need the general path (no real grids)
        plan = F.VoxelPlan(geom, structures, phis=phis, fill_bkg=True, smooth=1,
                           fft_y=1024, fft_z=1280, transform=tr,
                           real=False if opt == "shells" else None, **kw)
        plan.set_atoms()
        if opt == "shells":
            lower = np.array([0.0, 0.7, 1.4])
            upper = np.array([0.7, 1.4, 2.2])
            f_sh = np.stack([fv * (1.0 - 0.1 * k) for k in range(3)])
            avg = np.array([[0.02 + 0j], [0.019 + 0j], [0.018 + 0j]])
            plan.set_shells(geom.q, lower, upper, f_sh, avg)
        plan.execute()
        if opt == "graph":
            plan.capture_graph()
            plan.execute()
            plan.execute()
        outs[tr] = (plan.iq(), plan.counts(), plan.info())
        plan.close()
    (a, ca, ia), (b, cb, ib) = outs["fused"], outs["stockham"]
    assert (ia["fused_y"], ia["fused_z"]) == (1, 1)
    assert np.array_equal(ca, cb)
    assert rel_l2(a, b) <= RTOL
    if opt == "structs":
        ref = O.voxelgrid([(s[0], s[1]) for s in structures], 0.5, 0.15, 1.5,
                          phis, True, 1)
        assert rel_l2(a, ref["iq"]) <= RTOL
