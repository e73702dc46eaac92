"""Gather binning (gw_voxel_params.binning): the column transforms store
every slice's |F|^2 pixels and one pass per voxel line adds them in a fixed
order, against the float64 atomic binning and the float64 oracle: real and
general grids, fill/smoothing, several structures averaged and separate,
float64 sums and I(q) on request, graph replay, multi-q shells (which bin
atomically on a gather plan), and the plans it refuses.  Counts bit-exact;
intensities by normwise relative L2 <= 1e-5 against the oracle and 1e-6
between the two binnings; results bit-identical run to run where the
deposit is (one f value per structure)."""
import os

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from oracle import giwaxs_oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5
GEOM = (0.5, 0.15, 1.5)
PHIS = np.array([0.0, 11.0, 45.0, 90.0, 133.5, 170.0])


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(
        np.linalg.norm(np.asarray(b)), 1e-300)


def slab(kind, seed, size):
    rng = np.random.default_rng(seed)
    make = W.graphite_slab if kind == "C" else W.silicon_slab
    return make(size, rng, disp_sigma=0.05)[0]


def run(structures, fill, smooth, repeat=1, graph=False, sums=False, **kw):
    plan = F.VoxelPlan(F.VoxelGeometry(*GEOM), structures, phis=PHIS,
                       fill_bkg=fill, smooth=smooth, **kw)
    try:
        plan.set_atoms()
        plan.execute()
        if graph:
            plan.capture_graph()
        outs = []
        for _ in range(repeat):
            if graph or repeat > 1:
                plan.execute()
            outs.append(plan.iq32().copy())
        out = dict(iq=plan.iq().copy(), iq32=outs, counts=plan.counts(),
                   info=plan.info())
        if sums:
            out["sums"] = plan.sums().copy()
        return out
    finally:
        plan.close()


@pytest.mark.parametrize("kind", ["real", "general"])
@pytest.mark.parametrize("fill,smooth", [(False, 0), (True, 1.5)])
def test_gather_vs_atomic_and_oracle(kind, fill, smooth):
    xyz = slab("C", 31, (12.0, 11.0, 13.0))
    n = len(xyz)
    if kind == "real":
        fv = np.full(n, 6.0 + 0.2j)
    else:  # two elements of different phases: the general path
        fv = np.where(np.arange(n) % 3 == 0, 14.0 + 0.3j, 6.0 + 0.01j)
    s = [(xyz, fv, None)]
    ga = run(s, fill, smooth, repeat=3, sums=True, binning="gather")
    at = run(s, fill, smooth, binning="atomic", sums=True)
    auto = run(s, fill, smooth)  # a sum grid in L2: atomic
    assert ga["info"]["gather"] == 1 and at["info"]["gather"] == 0
    assert auto["info"]["gather"] == 0
    assert ga["info"]["real"] == (kind == "real")
    ref = O.voxelgrid([(xyz, fv)], *GEOM, PHIS, fill, smooth)
    assert np.array_equal(ga["counts"], ref["count"])
    assert rel_l2(ga["iq"], ref["iq"]) <= RTOL
    assert rel_l2(ga["iq"], at["iq"]) <= 1e-6
    assert rel_l2(ga["sums"], at["sums"]) <= 1e-6
    # the same bits on every execute where the deposit's shared-memory sums
    # are order-independent (one f value: every partial sum is k f); with
    # several f values a cell of three or more atoms rounds by arrival
    # order in float32, the binning adds nothing to that
    for x in ga["iq32"][1:]:
        if kind == "real":
            assert np.array_equal(x.view(np.uint32), ga["iq32"][0].view(np.uint32))
        else:
            assert rel_l2(x, ga["iq32"][0]) <= 1e-6
    # float32 I(q) within 2 ulps of the float64 I(q) rounded (both of the
    # last execute), zero together
    r32 = ga["iq"].astype(np.float32)
    i32 = ga["iq32"][-1]
    assert np.array_equal(i32 == 0, r32 == 0)
    ulps = np.abs(i32.view(np.int32).astype(np.int64) - r32.view(np.int32).astype(np.int64))
    assert ulps.max() <= 2


@pytest.mark.parametrize("average", [True, "separate"])
def test_gather_structures(average):
    a = slab("C", 32, (12.0, 11.0, 13.0))
    b = slab("Si", 33, (9.0, 14.0, 7.0))
    c = slab("C", 34, (13.0, 8.0, 10.0))
    s = [(a, np.full(len(a), 6.0 + 0j), None),
         (b, np.full(len(b), 14.1 + 0.4j), None),
         (c, np.full(len(c), 5.9 - 0.1j), None)]
    ga = run(s, True, 1.0, average=average, graph=True, repeat=2, binning="gather")
    at = run(s, True, 1.0, average=average, binning="atomic")
    assert ga["info"]["gather"] == 1
    assert np.array_equal(ga["counts"], at["counts"])
    assert rel_l2(ga["iq"], at["iq"]) <= 1e-6
    assert np.array_equal(ga["iq32"][0].view(np.uint32), ga["iq32"][1].view(np.uint32))
    if average is True:
        ref = O.voxelgrid([(x[0], x[1]) for x in s], *GEOM, PHIS, True, 1.0)
        assert rel_l2(ga["iq"], ref["iq"]) <= RTOL


def test_shells_bin_atomically_on_a_gather_plan():
    geom = F.VoxelGeometry(*GEOM)
    xyz = slab("C", 35, (12.0, 11.0, 13.0))
    fv = np.full(len(xyz), 6.0 + 0j)
    lower = np.array([0.0, 0.7, 1.4])
    upper = np.array([0.7, 1.4, 2.2])
    f_sh = np.stack([fv * (1.0 - 0.1 * k) for k in range(3)])
    avg = np.array([[0.02 + 0j], [0.019 + 0j], [0.018 + 0j]])
    outs = {}
    for binning in ("gather", "atomic"):
        plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=PHIS, fill_bkg=True,
                           smooth=1, real=False, binning=binning)
        plan.set_atoms()
        plan.set_shells(geom.q, lower, upper, f_sh, avg)
        plan.execute()
        outs[binning] = (plan.iq().copy(), plan.info()["gather"])
        plan.set_shells(None, None, None, None, None)
        plan.set_atoms()
        plan.execute()                 # shells cleared: gathers again
        outs[binning + "-plain"] = plan.iq().copy()
        plan.close()
    assert outs["gather"][1] == 1 and outs["atomic"][1] == 0
    assert rel_l2(outs["gather"][0], outs["atomic"][0]) <= 1e-12
    assert rel_l2(outs["gather-plain"], outs["atomic-plain"]) <= 1e-6


def test_plans_gather_refuses(monkeypatch):
    geom = F.VoxelGeometry(*GEOM)
    xyz = slab("C", 36, (10.0, 10.0, 10.0))
    fv = np.full(len(xyz), 6.0 + 0j)
    for kw in (dict(accum="kahan32"), dict(mode="plain")):
        with pytest.raises(N.GwError) as e:
            F.VoxelPlan(geom, [(xyz, fv, None)], phis=PHIS, binning="gather", **kw)
        assert e.value.status == N.GW_ERR_ARG
        # auto: the atomic binning (and for so small a grid anyway)
        p = F.VoxelPlan(geom, [(xyz, fv, None)], phis=PHIS, **kw)
        assert p.info()["gather"] == 0
        p.close()
    # a pixel store over the budget
    monkeypatch.setenv("GW_GATHER_MAX_MB", "0")
    with pytest.raises(N.GwError):
        F.VoxelPlan(geom, [(xyz, fv, None)], phis=PHIS, binning="gather")
    monkeypatch.delenv("GW_GATHER_MAX_MB")
    assert os.environ.get("GW_GATHER_MAX_MB") is None


def test_chunked_result_copy(monkeypatch):
    """The float64 I(q) made in runs of lines, each copied to the (resident)
    host array as soon as it is made, is the one-launch result bit for bit,
    heavy lines (a block each) split between runs included."""
    xyz = slab("C", 37, (12.0, 11.0, 13.0))
    fv = np.full(len(xyz), 6.0 + 0.2j)
    phis = np.arange(0.0, 180.0, 0.5)  # about 180 entries on the axis line
    plan = F.VoxelPlan(F.VoxelGeometry(*GEOM), [(xyz, fv, None)], phis=phis,
                       fill_bkg=True, smooth=1.0, binning="gather")
    outs = {}
    try:
        plan.set_atoms()
        for k in ("1", "3", "8", "16"):
            monkeypatch.setenv("GW_IQ_CHUNKS", k)
            plan.execute()
            out = np.full((plan.Qc,) * 3, -1.0)  # every page resident
            plan.iq(out=out)
            outs[k] = out
        info = plan.info()
        counts = plan.counts()
    finally:
        plan.close()
    assert info["gather"] == 1 and info["real"] == 1
    assert info["heavy_lines"] > 0
    for k in ("3", "8", "16"):
        assert np.array_equal(outs[k].view(np.uint64), outs["1"].view(np.uint64)), k
    assert not outs["1"][counts == 0].any()
    assert (outs["1"] >= 0).all()
