"""GPU voxel stage against the oracle (and the reference fixtures).

Tolerances: bin/voxel indices and counts are compared bit-exact; intensities
(the float32 transform) by normwise relative L2 error <= 1e-5 against the
float64 oracle, the bar the forward path is specified to."""
import numpy as np
import pytest

from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import comparison
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(
        np.linalg.norm(np.asarray(b)), 1e-300)


def gpu_run(geom, structures, phis, fill, smooth, **kw):
    plan = F.VoxelPlan(geom, structures, phis=phis, fill_bkg=fill,
                       smooth=smooth, **kw)
    plan.set_atoms()
    plan.execute()
    out = dict(iq=plan.iq(), counts=plan.counts(), sums=plan.sums(),
               info=plan.info(), plan=plan)
    return out


def small_case(seed=0, size=(12.0, 11.0, 13.0)):
    rng = np.random.default_rng(seed)
    xyz, _ = W.graphite_slab(size, rng, disp_sigma=0.05)
    return xyz, np.full(len(xyz), 6.0 + 0j)


MODES = [("plain", False, 0), ("fill", True, 0), ("smooth", False, 2),
         ("fillsmooth", True, 1)]


@pytest.mark.parametrize("name,fill,smooth", MODES)
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_small_slices_vs_oracle(name, fill, smooth, mode):
    xyz, fv = small_case()
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.array([0.0, 17.0, 45.0, 90.0, 133.5])
    ref = O.voxelgrid([(xyz, fv)], 0.5, 0.15, 1.5, phis, fill, smooth)
    got = gpu_run(geom, [(xyz, fv, None)], phis, fill, smooth, mode=mode)
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["sums"], ref["sum"]) <= RTOL
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL


@pytest.mark.parametrize("name,fill,smooth", MODES)
def test_reference_fixture_slices(name, fill, smooth):
    """Against the reference's own rotate_project_fft_coords output."""
    d = golden("golden_slices.npz")
    xyz = d["coords"]
    fv = np.full(len(xyz), 6.0 + 0j)
    geom = F.VoxelGeometry(float(d["r"]), float(d["dq"]), float(d["max_q"]))
    got = gpu_run(geom, [(xyz, fv, None)], d["phis"], fill, smooth)
    lo, hi = geom.crop_lo, geom.crop_hi + 1
    ref_c = d["count_" + name][lo:hi, lo:hi, lo:hi]
    ref_s = d["sum_" + name][lo:hi, lo:hi, lo:hi]
    assert np.array_equal(got["counts"], ref_c)
    assert rel_l2(got["sums"], ref_s) <= RTOL


@pytest.mark.parametrize("name", ["plain", "fillsmooth"])
def test_reference_fixture_driver(name):
    d = golden("golden_voxel.npz")
    xyz = d["coords"]
    fill, smooth = (False, 0) if name == "plain" else (True, 1)
    iq, qx, qy, qz = comparison.voxelgridmaker_fitting(
        xyz, np.array(["C"] * len(xyz)), float(d["r"]), float(d["dq"]),
        float(d["max_q"]), 10000, fill_bkg=fill, smooth=smooth)
    assert np.array_equal(qx, d["qx"])
    assert rel_l2(iq, d["iq_" + name]) <= RTOL


def test_deposit_indices_bit_exact():
    xyz, fv = small_case(3, (20.0, 17.0, 15.0))
    geom = F.VoxelGeometry(0.3, 0.1, 1.5)
    phis = np.linspace(0, 179, 23)
    got = gpu_run(geom, [(xyz, fv, None)], phis, False, 0)
    for k, phi in enumerate(phis):
        y, z = got["plan"].debug_deposit(k)
        _, info = O.project_slice(xyz, fv, phi, geom.grid_size, 0.3, 0j, 1, 1,
                                  1, False, 0)
        ok = info["valid"]
        ry = np.full(len(xyz), -1)
        rz = np.full(len(xyz), -1)
        ry[ok], rz[ok] = info["y_idx"], info["z_idx"]
        assert np.array_equal(y, ry) and np.array_equal(z, rz), phi


def test_graphite_50A_reduced_phis():
    """graphite-50A geometry (g=699) on 8 of its 180 slices."""
    xyz, el, _ = W.structures("graphite-50A")[0]
    fv = F.element_f_values(el, 10000.0)
    w = W.WORKLOADS["graphite-50A"]
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = W.phis_linspace(180)[::23]
    ref = O.voxelgrid([(xyz, fv)], w["r"], w["dq"], w["max_q"], phis, False, 0)
    got = gpu_run(geom, [(xyz, fv, None)], phis, False, 0)
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL


def test_si_100A_fill_smooth_reduced_phis():
    """si-100A geometry (g=1257, fill_bkg, smooth=2) on 3 slices."""
    xyz, el, _ = W.structures("si-100A")[0]
    fv = F.element_f_values(el, 12000.0)
    w = W.WORKLOADS["si-100A"]
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = np.array([0.0, 33.5, 121.0])
    ref = O.voxelgrid([(xyz, fv)], w["r"], w["dq"], w["max_q"], phis, True, 2)
    got = gpu_run(geom, [(xyz, fv, None)], phis, True, 2)
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL


def test_full_size_counts_graphite_50A():
    """All 180 slices: the count grid (geometry only) bit-exact against the
    oracle's binning tables."""
    xyz, el, _ = W.structures("graphite-50A")[0]
    fv = F.element_f_values(el, 10000.0)
    w = W.WORKLOADS["graphite-50A"]
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = W.phis_linspace(180)
    got = gpu_run(geom, [(xyz, fv, None)], phis, False, 0)
    q = geom.q
    cnt = np.zeros((len(q),) * 3)
    for phi in phis:
        hx, hy, vz = O.slice_axes(geom.grid_size, w["r"], phi)
        vm, hm, iy, ix, iz = O.bin_indices(hx, hy, vz, q, q, q)
        IY = np.repeat(iy, len(iz))
        IX = np.repeat(ix, len(iz))
        IZ = np.tile(iz, len(iy))
        np.add.at(cnt, (IY, IX, IZ), 1.0)
    lo, hi = geom.crop_lo, geom.crop_hi + 1
    assert np.array_equal(got["counts"], cnt[lo:hi, lo:hi, lo:hi])
    assert np.all(np.isfinite(got["iq"])) and got["iq"].max() > 0


def test_multi_structure_average_and_kahan():
    structs = [small_case(s, (10.0 + s, 11.0, 9.0 + 2 * s)) for s in range(3)]
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.array([0.0, 30.0, 75.0, 140.0])
    ref = O.voxelgrid([(x, f) for x, f in structs], 0.5, 0.15, 1.5, phis,
                      False, 1)
    items = [(x, f, None) for x, f in structs]
    got = gpu_run(geom, items, phis, False, 1)
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL
    got_k = gpu_run(geom, items, phis, False, 1, accum="kahan32")
    assert rel_l2(got_k["iq"], ref["iq"]) <= RTOL


def test_graph_replay_matches_eager():
    xyz, fv = small_case()
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.linspace(0, 170, 9)
    plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=phis, fill_bkg=True,
                       smooth=1)
    plan.set_atoms()
    plan.execute()
    eager = plan.iq()
    plan.capture_graph()
    for _ in range(2):
        plan.execute()
        assert rel_l2(plan.iq(), eager) <= 1e-12


@pytest.mark.parametrize("name,n_phi,force,expect_m", [
    ("graphite-50A", 2, 0, 1536), ("graphite-50A", 2, 2048, 2048),
    ("si-100A", 1, 0, 2560), ("si-100A", 1, 4096, 4096),
    ("lamellar-200A", 1, 0, 5120), ("lamellar-200A", 1, 8192, 8192)])
def test_plain_mode_large_transforms(name, n_phi, force, expect_m):
    """Plain (full-grid) mode at full workload grid sizes: the automatic
    1536-, 2560- and 5120-point transforms and forced 2048-, 4096- and
    8192-point ones against the oracle's numpy fftn."""
    structs = W.structures(name)
    xyz, el, _ = structs[0]
    w = W.WORKLOADS[name]
    fv = F.element_f_values(el, w["energy"])
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = np.array([0.0, 61.0])[:n_phi]
    ref = O.voxelgrid([(xyz, fv)], w["r"], w["dq"], w["max_q"], phis,
                      w["fill_bkg"], w["smooth"])
    got = gpu_run(geom, [(xyz, fv, None)], phis, w["fill_bkg"], w["smooth"],
                  mode="plain", fft_y=force, fft_z=force)
    assert got["info"]["My"] == expect_m
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL
    bat = gpu_run(geom, [(xyz, fv, None)], phis, w["fill_bkg"], w["smooth"])
    assert rel_l2(bat["iq"], ref["iq"]) <= RTOL


@pytest.mark.parametrize("name,n_phi", [("graphite-50A", 6), ("si-100A", 4),
                                        ("graphite-64", 3)])
def test_deposit_window_bit_exact(name, n_phi):
    """The fused deposit (z-sorted atoms, per-slice shift and floor division,
    shared-memory accumulation path) equals the oracle's np.add.at grid on
    the transformed window, bit for bit (f = Z sums are exact in float32)."""
    structs = W.structures(name)[:2]
    w = W.WORKLOADS[name]
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    phis = np.linspace(0, 179, n_phi)
    items = [(x, F.element_f_values(e, w["energy"]), None) for x, e, _ in structs]
    plan = F.VoxelPlan(geom, items, phis=phis, fill_bkg=w["fill_bkg"],
                       smooth=w["smooth"])
    plan.set_atoms()
    plan.execute()
    g = geom.grid_size
    for t, (xyz, fv, _) in enumerate(items):
        for k, phi in enumerate(phis):
            win, z_lo, y_lo = plan.debug_window(t * len(phis) + k)
            grid, _ = O.project_slice(xyz, fv, phi, g, w["r"], 0j, 1, 1, 1,
                                      False, 0)
            zi = (z_lo + np.arange(win.shape[0])) % g
            yi = (y_lo + np.arange(win.shape[1])) % g
            ref = grid[np.ix_(zi, yi)]
            assert np.array_equal(win.astype(np.complex128), ref), (t, phi)
            assert np.abs(ref).sum() == np.abs(grid).sum()  # window holds all


FFT_SIZES = [128, 256, 384, 512, 640, 768, 1024, 1280, 1536, 2048, 2560,
             3072, 4096, 5120, 6144, 8192]


@pytest.mark.parametrize("m", FFT_SIZES)
def test_every_transform_length(m):
    """Each supported chirp-z length (2^k, 3*2^k, 5*2^k: radix-16/8/4/2
    passes plus a radix-3 or radix-5 pass) forced on both axes of a small
    smoothed case gives the oracle's I(q)."""
    xyz, fv = small_case(seed=4)
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.array([0.0, 31.0, 90.0, 151.0])
    ref = O.voxelgrid([(xyz, fv)], 0.5, 0.15, 1.5, phis, False, 1.5)
    got = gpu_run(geom, [(xyz, fv, None)], phis, False, 1.5, fft_y=m, fft_z=m)
    assert (got["info"]["My"], got["info"]["Mz"]) == (m, m)
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL


def test_autotuned_plan_vs_oracle(tmp_path, monkeypatch):
    """A tuned plan (lengths and batch chosen by timing) gives the oracle's
    I(q); the choice is cached for the next plan of the same shape."""
    monkeypatch.setenv("GIWAXSIM_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    xyz, fv = small_case(seed=6)
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    phis = np.linspace(0.0, 180.0, 24, endpoint=False)
    ref = O.voxelgrid([(xyz, fv)], 0.5, 0.15, 1.5, phis, False, 1.5)
    got = gpu_run(geom, [(xyz, fv, None)], phis, False, 1.5, tune=True)
    plan = got["plan"]
    assert set(plan.tuned) == {"fft_y", "fft_z", "batch_slices", "transform",
                               "block_variant", "binning"}
    assert got["info"]["gather"] == (plan.tuned["binning"] == "gather")
    assert (got["info"]["My"], got["info"]["Mz"]) == (plan.tuned["fft_y"],
                                                      plan.tuned["fft_z"])
    # the families the plan runs: fused where asked for, else Stockham
    fam = tuple("fused" if f else "stockham"
                for f in (got["info"]["fused_y"], got["info"]["fused_z"]))
    assert fam == tuple("fused" if t == "fused" else "stockham"
                        for t in plan.tuned["transform"])
    assert np.array_equal(got["counts"], ref["count"])
    assert rel_l2(got["iq"], ref["iq"]) <= RTOL
    assert (tmp_path / "t.json").exists()
