"""The oracle against outputs of the reference itself (tests/golden, made by
tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import giwaxs_oracle as O
from tests.conftest import golden


def test_rotate_coords_z_bits():
    d = golden("golden_rotation.npz")
    for phi, ref in zip(d["phis"], d["rot"]):
        got = O.rotate_coords_z(d["coords"], phi)
        assert np.array_equal(got, ref), phi


def test_detector_rotation_chain_bits():
    d = golden("golden_rotation.npz")
    x0, y0, z0, _, _ = O.make_detector(2.5, 9, 2.5, 7)
    for ang, ref in zip(d["det_angles"], d["det_rot"]):
        x, y, z = O.rotate_about(x0, y0, z0, "psi", ang[0])
        x, y, z = O.rotate_about(x, y, z, "phi", ang[1])
        x, y, z = O.rotate_about(x, y, z, "theta", ang[2])
        assert np.array_equal(np.stack([x, y, z]), ref), ang


def test_floor_division_is_exact_real_floor():
    from fractions import Fraction
    import math
    d = golden("golden_floordiv.npz")
    assert np.array_equal(d["a"] // d["b"], d["q"])
    sub = slice(0, None, 7)
    exact = [math.floor(Fraction(float(a)) / Fraction(float(b)))
             for a, b in zip(d["a"][sub], d["b"][sub])]
    assert np.array_equal(np.array(exact, dtype=np.float64), d["q"][sub])


def test_collapse_lengths_bits():
    d = golden("golden_collapse.npz")
    for phi, hor, ver, ref in zip(d["phi"], d["hor"], d["ver"], d["lengths"]):
        got = O.rectangular_collapse_lengths(d["x"], hor, ver, phi)
        assert np.array_equal(got, ref), (phi, hor, ver)


@pytest.mark.parametrize("mode,fill,smooth", [
    ("plain", False, 0), ("fill", True, 0), ("smooth", False, 2),
    ("fillsmooth", True, 1)])
def test_slices_sum_count(mode, fill, smooth):
    d = golden("golden_slices.npz")
    xyz, q, g, r = d["coords"], d["q"], int(d["g"]), float(d["r"])
    fv = np.full(len(xyz), 6.0 + 0j)
    xb, yb, zb, avg = O.structure_constants(xyz, fv, r)
    qn = len(q)
    vs, vc = np.zeros((qn,) * 3), np.zeros((qn,) * 3)
    for phi in d["phis"]:
        grid, _ = O.project_slice(xyz, fv, phi, g, r, avg, xb, yb, zb, fill,
                                  smooth)
        hx, hy, vz = O.slice_axes(g, r, phi)
        O.bin_slice(O.slice_intensity(grid), hx, hy, vz, q, q, q, vs, vc)
    assert np.array_equal(vc, d["count_" + mode])
    ref = d["sum_" + mode]
    assert np.linalg.norm(vs - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("mode,fill,smooth", [("plain", False, 0),
                                              ("fillsmooth", True, 1)])
def test_voxel_driver(mode, fill, smooth):
    d = golden("golden_voxel.npz")
    xyz = d["coords"]
    fv = np.full(len(xyz), 6.0 + 0j)
    out = O.voxelgrid([(xyz, fv)], float(d["r"]), float(d["dq"]),
                      float(d["max_q"]), None, fill, smooth)
    for k in ("qx", "qy", "qz"):
        assert np.array_equal(out[k], d[k])
    ref = d["iq_" + mode]
    assert out["iq"].shape == ref.shape
    assert np.linalg.norm(out["iq"] - ref) <= 1e-12 * np.linalg.norm(ref)


def test_detector_driver():
    v = golden("golden_voxel.npz")
    d = golden("golden_detector.npz")
    iq, qx, qy, qz = v["iq_plain"], v["qx"], v["qy"], v["qz"]
    det, h, vv = O.detector(iq, qx, qy, qz, 21, 1.2, (90.0, 30.0, 10.0),
                            ("psi", "phi", "theta"), np.linspace(0, 180, 7),
                            None, np.array([0.0, 20.0]), None,
                            np.array([0.0, 5.0]), None, mirror=True)
    assert np.array_equal(h, d["det_h"]) and np.array_equal(vv, d["det_v"])
    assert np.linalg.norm(det - d["det_sum"]) <= 1e-13 * np.linalg.norm(
        d["det_sum"])
    det2, _, _ = O.detector(iq, qx, qy, qz, 16, 1.2, (0.0, 0.0, 0.0),
                            ("None",) * 3, np.linspace(0, 90, 10), None,
                            np.array([0.0]), None, np.array([0.0]), None, True)
    assert np.linalg.norm(det2 - d["det_sum2"]) <= 1e-13 * np.linalg.norm(
        d["det_sum2"])
    x0, y0, z0, _, _ = O.make_detector(1.2, 21, 1.2, 21)
    for ang, ref in zip(d["single_angles"], d["singles"]):
        x, y, z = O.rotate_psi_phi_theta(x0, y0, z0, *ang)
        assert np.array_equal(O.intersect_detector(iq, qx, qy, qz, x, y, z),
                              ref)


def test_mirror():
    d = golden("golden_mirror.npz")
    for shp in [(7, 9), (8, 6), (7, 6), (8, 9)]:
        got = O.mirror_vertical_horizontal(d["in_%dx%d" % shp])
        assert np.array_equal(got, d["out_%dx%d" % shp])


def test_f0_and_downselect():
    d = golden("golden_f0.npz")
    q = d["q"]
    got = O.add_f0_q_3d(d["grid"], q, q, q, "C")
    assert np.allclose(got, d["f0"], rtol=1e-14, atol=0)
    sub, x, _, _ = O.downselect_voxelgrid(d["grid"], q, q, q, 1.1)
    assert np.array_equal(sub, d["ds_grid"]) and np.array_equal(x, d["ds_x"])


SLAB_CASES = ["pm6", "graphite", "graphite_odd", "triclinic"]


def _slab_sha(coords, els):
    import hashlib
    return (hashlib.sha256(np.ascontiguousarray(coords, dtype=np.float64).tobytes()).hexdigest(),
            hashlib.sha256("".join(np.asarray(els).tolist()).encode()).hexdigest())


@pytest.mark.parametrize("name", SLAB_CASES)
def test_slabmaker_vs_reference(name):
    """The oracle's slab (and the package's cell vectors) against the
    reference's slabmaker_fitting, every coordinate bit for bit."""
    from giwaxsim_gb300.tools.utilities import calc_real_space_abc
    d = golden("golden_slab.npz")
    vecs = calc_real_space_abc(*d[name + "_cellp"])
    coords, els = O.slabmaker(d[name + "_cell_xyz"], d[name + "_cell_el"], vecs,
                              tuple(d[name + "_size"]))
    assert len(coords) == int(d[name + "_n"])
    assert np.array_equal(coords[:8], d[name + "_head"])
    assert _slab_sha(coords, els) == (str(d[name + "_sha"]), str(d[name + "_el_sha"]))


@pytest.mark.parametrize("name", ["plain", "fillsmooth"])
def test_multi_q_vs_reference(name):
    """generate_voxel_grid_low_mem with aff_num_qs > 1, bit for bit."""
    d = golden("golden_multiq.npz")
    r = O.voxelgrid_multi_q(d["coords"], d["elements"], {"C": 0j, "O": 0j},
                            float(d["r"]), float(d["dq"]), float(d["max_q"]),
                            int(d[name + "_K"]), fill_bkg=bool(d[name + "_fill"]),
                            smooth=int(d[name + "_smooth"]))
    assert np.array_equal(r["q"], d["q"])
    assert np.array_equal(r["iq"], d[name + "_iq"])
    # shells cover (0, max_q_diag]: the centre voxel and the cube's corners
    # lie in none, every other voxel in exactly one
    n_in = sum(m.astype(int) for m in r["masks"])
    qx, qy, qz = np.meshgrid(r["q"], r["q"], r["q"])
    qr = np.sqrt(qx ** 2 + qy ** 2 + qz ** 2)
    assert n_in.max() == 1
    assert np.array_equal(n_in == 1, (qr > 0) & (qr <= r["q"][-1]))


@pytest.mark.parametrize("name", ["pad", "nopad"])
def test_shift_peak_vs_reference(name):
    """shift_peak (polar warp, pi-pi padding, inverse warp), bit for bit."""
    d = golden("golden_shift.npz")
    out = O.shift_peak(d["img"].copy(), d["det_h"], d["det_v"],
                       float(d[name + "_pw"]), tuple(d[name + "_pr"]))
    assert np.array_equal(out, d[name + "_out"])


@pytest.mark.parametrize("name", ["pad", "nopad"])
def test_shift_peak_maps_vs_reference(name):
    """The product's fixed shift_peak maps (host geometry, applied here in
    numpy) reproduce the reference's output to rounding."""
    from giwaxsim_gb300.tools.comparison import shift_peak_maps
    d = golden("golden_shift.npz")
    img = d["img"]
    m = shift_peak_maps(d["det_h"], d["det_v"], img.shape,
                        float(d[name + "_pw"]), tuple(d[name + "_pr"]))

    def apply(idx, w, v):
        vals = np.where(idx >= 0, v[np.maximum(idx, 0)], 0.0)
        return sum(vals[:, k] * w[:, k] for k in range(4))

    polar = apply(m["p_idx"], m["p_w"], img.ravel()).reshape(m["n_t"], m["n_r"])
    z = np.where(polar == 0, 0.0, polar[:, m["col_src"]])
    out = apply(m["q_idx"], m["q_w"], z.ravel()).reshape(img.shape)
    ref = d[name + "_out"]
    assert np.abs(out - ref).max() <= 1e-14 * np.abs(ref).max()


def test_threaded_crop_oracle_equals_serial():
    """The threaded, crop-only oracle the bench and the full-size GPU test
    use gives the serial oracle's counts exactly and its sums to rounding."""
    from giwaxsim_gb300 import workloads as W
    rng = np.random.default_rng(3)
    xyz, _ = W.graphite_slab((12.0, 11.0, 13.0), rng, disp_sigma=0.05)
    fv = np.full(len(xyz), 6.0 + 0j)
    phis = np.linspace(0, 180, 20, endpoint=False)
    a = O.voxelgrid([(xyz, fv)], 0.5, 0.15, 1.5, phis, True, 1.5)
    b = O.voxelgrid_crop_threaded(xyz, fv, 0.5, 0.15, 1.5, phis, True, 1.5, workers=4)
    assert np.array_equal(a["count"], b["count"])
    assert np.abs(a["iq"] - b["iq"]).max() <= 1e-12 * np.abs(a["iq"]).max()
