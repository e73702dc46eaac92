"""The real-grid path (gw_voxel_params.real_grids: every structure's atom f
values real multiples of one complex value, so each slice grid is that
phase times a real grid; two window rows share one row transform and only
the columns ky >= 0 are transformed, the others binned from their mirror)
against the general path and the float64 oracle: one element with a real
and with a complex f, occupancies, f values of both signs, fill/smoothing,
Kahan float32 accumulation, several structures averaged and separate,
graph replay.  Counts bit-exact; intensities by normwise relative L2 <=
1e-5.  Plans that do not allow it (several elements, the bilinear deposit,
multi-q shells, other f values uploaded later) keep or ask for the general
path."""
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


def run(geom, structures, phis, fill, smooth, graph=False, **kw):
    plan = F.VoxelPlan(geom, structures, phis=phis, fill_bkg=fill,
                       smooth=smooth, **kw)
    try:
        plan.set_atoms()
        plan.execute()
        if graph:
            plan.capture_graph()
            plan.execute()
            plan.execute()
        return dict(iq=plan.iq().copy(), counts=plan.counts(), info=plan.info())
    finally:
        plan.close()


def slab(kind, seed, size):
    rng = np.random.default_rng(seed)
    make = W.graphite_slab if kind == "C" else W.silicon_slab
    xyz, _ = make(size, rng, disp_sigma=0.05)
    return xyz


GEOM = (0.5, 0.15, 1.5)
PHIS = np.array([0.0, 11.0, 45.0, 90.0, 133.5, 170.0])


@pytest.mark.parametrize("f", [6.0 + 0j, 14.2 + 0.37j, -3.0 - 4.0j])
@pytest.mark.parametrize("fill,smooth", [(False, 0), (True, 1.5)])
def test_real_vs_general_and_oracle(f, fill, smooth):
    xyz = slab("C", 21, (12.0, 11.0, 13.0))
    fv = np.full(len(xyz), f)
    geom = F.VoxelGeometry(*GEOM)
    ref = O.voxelgrid([(xyz, fv)], *GEOM, PHIS, fill, smooth)
    re = run(geom, [(xyz, fv, None)], PHIS, fill, smooth)
    ge = run(geom, [(xyz, fv, None)], PHIS, fill, smooth, real=False)
    assert re["info"]["real"] == 1 and ge["info"]["real"] == 0
    assert np.array_equal(re["counts"], ref["count"])
    assert np.array_equal(ge["counts"], ref["count"])
    assert rel_l2(re["iq"], ref["iq"]) <= RTOL
    assert rel_l2(re["iq"], ge["iq"]) <= RTOL


def test_occupancies_and_signs():
    """Weights (occupancies) and f values of both signs along one phase
    still give real grids."""
    xyz = slab("Si", 22, (11.0, 12.0, 10.0))
    rng = np.random.default_rng(3)
    fv = (14.0 + 0.3j) * np.where(rng.random(len(xyz)) < 0.3, -0.5, 1.0)
    w = rng.uniform(0.2, 1.0, len(xyz))
    geom = F.VoxelGeometry(*GEOM)
    re = run(geom, [(xyz, fv, w)], PHIS, True, 1.0)
    assert re["info"]["real"] == 1
    ref = O.voxelgrid([(xyz, fv * w)], *GEOM, PHIS, True, 1.0)
    assert np.array_equal(re["counts"], ref["count"])
    assert rel_l2(re["iq"], ref["iq"]) <= RTOL


@pytest.mark.parametrize("opt", ["kahan32", "structs", "separate", "graph",
                                 "batch"])
def test_real_options_vs_general(opt):
    geom = F.VoxelGeometry(*GEOM)
    xyz = slab("C", 23, (12.0, 11.0, 13.0))
    structures = [(xyz, np.full(len(xyz), 6.0 + 0j), None)]
    kw, graph = {}, False
    if opt == "kahan32":
        kw["accum"] = "kahan32"
    elif opt in ("structs", "separate"):
        # each structure its own phase
        x2 = slab("Si", 24, (9.0, 14.0, 7.0))
        x3 = slab("C", 25, (13.0, 8.0, 10.0))
        structures += [(x2, np.full(len(x2), 14.1 + 0.4j), None),
                       (x3, np.full(len(x3), 5.9 - 0.1j), None)]
        if opt == "separate":
            kw["average"] = "separate"
    elif opt == "graph":
        graph = True
    elif opt == "batch":
        kw["batch_slices"] = 4   # a partial last batch
    re = run(geom, structures, PHIS, True, 1.0, graph=graph, **kw)
    ge = run(geom, structures, PHIS, True, 1.0, graph=graph, real=False, **kw)
    assert re["info"]["real"] == 1
    assert np.array_equal(re["counts"], ge["counts"])
    if opt == "separate":
        for a, b in zip(re["iq"], ge["iq"]):
            assert rel_l2(a, b) <= RTOL
    else:
        assert rel_l2(re["iq"], ge["iq"]) <= RTOL
    if opt == "structs":
        ref = O.voxelgrid([(s[0], s[1]) for s in structures], *GEOM, PHIS,
                          True, 1.0)
        assert rel_l2(re["iq"], ref["iq"]) <= RTOL


def test_larger_grid_vs_oracle():
    """A finer grid (r = 0.25 A, dq = 0.05 1/A, max q 3): longer windows
    and bands, several batches."""
    xyz = slab("Si", 26, (16.0, 22.0, 18.0))
    fv = np.full(len(xyz), 14.0 + 0.2j)
    geom = F.VoxelGeometry(0.25, 0.05, 3.0)
    phis = np.linspace(0.0, 180.0, 10, endpoint=False)
    re = run(geom, [(xyz, fv, None)], phis, True, 1.0)
    assert re["info"]["real"] == 1
    ref = O.voxelgrid([(xyz, fv)], 0.25, 0.05, 3.0, phis, True, 1.0)
    assert np.array_equal(re["counts"], ref["count"])
    assert rel_l2(re["iq"], ref["iq"]) <= RTOL


def test_plans_that_keep_the_general_path():
    geom = F.VoxelGeometry(*GEOM)
    xyz = slab("C", 27, (10.0, 10.0, 10.0))
    n = len(xyz)
    carbon, silicon = 6.0 + 0.01j, 14.0 + 0.3j  # different phases
    mixed = np.where(np.arange(n) % 3 == 0, silicon, carbon)
    out = run(geom, [(xyz, mixed, None)], PHIS, False, 0)
    assert out["info"]["real"] == 0
    ref = O.voxelgrid([(xyz, mixed)], *GEOM, PHIS, False, 0)
    assert rel_l2(out["iq"], ref["iq"]) <= RTOL
    with pytest.raises(ValueError):
        F.VoxelPlan(geom, [(xyz, mixed, None)], phis=PHIS, real=True)
    fv = np.full(n, 6.0 + 0j)
    assert run(geom, [(xyz, fv, None)], PHIS, False, 0,
               deposit="bilinear")["info"]["real"] == 0
    assert run(geom, [(xyz, fv, None)], PHIS, False, 0,
               transform="fused", fft_y=1024, fft_z=1024)["info"]["real"] == 0
    # one atom: zero extents, no finite average voxel f to take the phase of
    one = np.array([[1.3, -0.4, 2.2]])
    with np.errstate(divide="ignore", invalid="ignore"):
        assert run(geom, [(one, np.array([6.0 + 2.0j]), None)], PHIS, False, 0,
                   f0_element=None)["info"]["real"] == 0
        with pytest.raises(ValueError):
            F.VoxelPlan(geom, [(one, np.array([6.0 + 2.0j]), None)], phis=PHIS,
                        f0_element=None, real=True)
    plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=PHIS)
    try:
        assert plan.info()["real"] == 1
        plan.set_atoms()
        with pytest.raises(N.GwError) as e:
            plan.set_shells(geom.q, np.array([0.0]), np.array([3.0]),
                            fv[None, :], np.ones((1, 1), complex))
        assert e.value.status == N.GW_ERR_STATE
        # other f values on the same plan are refused on the host
        with pytest.raises(ValueError):
            plan.set_atoms(plan.xyz, mixed.astype(np.complex64).view(np.float32))
        # a real multiple of the plan's phase is accepted
        plan.set_atoms(plan.xyz, (2.0 * fv).astype(np.complex64).view(np.float32))
        plan.execute()
    finally:
        plan.close()
