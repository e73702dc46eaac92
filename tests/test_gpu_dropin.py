"""The reference's per-slice and helper entry points (drop-in signatures,
shared memory by name) on the GPU, against the oracle and the reference
fixtures; and the config-file driver."""
import os

import numpy as np
import pytest

from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import detector as D
from giwaxsim_gb300.tools import utilities as U
from giwaxsim_gb300.tools import voxelgrids as V
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def shm_pair(qn):
    s, c = U.create_shared_array((qn,) * 3), U.create_shared_array((qn,) * 3)
    for m in (s, c):
        np.ndarray((qn,) * 3, dtype=np.float64, buffer=m.buf)[:] = 0
    return s, c


def read(m, qn):
    return np.ndarray((qn,) * 3, dtype=np.float64, buffer=m.buf).copy()


def free(*ms):
    for m in ms:
        m.close()
        m.unlink()


@pytest.mark.parametrize("fill,smooth", [(False, 0), (True, 1), (False, 2)])
def test_rotate_project_fft_coords(fill, smooth):
    d = golden("golden_slices.npz")
    xyz, q, g, r = d["coords"], d["q"], int(d["g"]), float(d["r"])
    fv = np.full(len(xyz), 6.0 + 0j)
    xb, yb, zb, avg = O.structure_constants(xyz, fv, r)
    qn = len(q)
    s, c = shm_pair(qn)
    try:
        for phi in d["phis"]:
            V.rotate_project_fft_coords((xyz, fv, phi, g, r, avg, xb, yb, zb,
                                         fill, smooth, q, q, q, s.name, c.name))
        mode = {(False, 0): "plain", (True, 1): "fillsmooth",
                (False, 2): "smooth"}[(fill, smooth)]
        assert np.array_equal(read(c, qn), d["count_" + mode])
        assert rel_l2(read(s, qn), d["sum_" + mode]) <= RTOL
    finally:
        free(s, c)


def test_process_file2():
    d = golden("golden_slices.npz")
    xyz, q, g, r = d["coords"], d["q"], int(d["g"]), float(d["r"])
    fv = np.full(len(xyz), 6.0 + 0j)
    qn = len(q)
    s, c = shm_pair(qn)
    rs, rc = np.zeros((qn,) * 3), np.zeros((qn,) * 3)
    try:
        for phi in d["phis"]:
            grid, _ = O.project_slice(xyz, fv, phi, g, r, 0j, 1, 1, 1, False, 0)
            iq2 = O.slice_intensity(grid)
            hx, hy, vz = O.slice_axes(g, r, phi)
            V.process_file2(iq2, hx, hy, vz, q, q, q, s.name, c.name)
            O.bin_slice(iq2, hx, hy, vz, q, q, q, rs, rc)
        assert np.array_equal(read(c, qn), rc)
        assert rel_l2(read(s, qn), rs) <= 1e-12
    finally:
        free(s, c)


def test_helpers_match_reference_fixtures():
    m = golden("golden_mirror.npz")
    for shp in [(7, 9), (8, 6), (7, 6), (8, 9)]:
        assert np.array_equal(D.mirror_vertical_horizontal(m["in_%dx%d" % shp]),
                              m["out_%dx%d" % shp])
    f = golden("golden_f0.npz")
    q = f["q"]
    assert np.allclose(V.add_f0_q_3d(f["grid"], q, q, q, "C"), f["f0"],
                       rtol=1e-13, atol=0)
    sub, x, _, _ = V.downselect_voxelgrid(f["grid"], q, q, q, 1.1)
    assert np.array_equal(sub, f["ds_grid"]) and np.array_equal(x, f["ds_x"])
    cl = golden("golden_collapse.npz")
    for phi, hor, ver, ref in zip(cl["phi"], cl["hor"], cl["ver"], cl["lengths"]):
        assert np.array_equal(V.rectangular_collapse_lengths(cl["x"], hor, ver, phi),
                              ref), (phi, hor, ver)


def test_detector_pieces_bit_exact():
    v = golden("golden_voxel.npz")
    d = golden("golden_detector.npz")
    iq, qx, qy, qz = v["iq_plain"], v["qx"], v["qy"], v["qz"]
    x0, y0, z0, _, _ = D.make_detector(1.2, 21, 1.2, 21)
    for ang, ref in zip(d["single_angles"], d["singles"]):
        x, y, z = D.rotate_psi_phi_theta(x0, y0, z0, *ang)
        assert np.array_equal(D.intersect_detector(iq, qx, qy, qz, x, y, z), ref)
    r = golden("golden_rotation.npz")
    dx, dy, dz, _, _ = D.make_detector(2.5, 9, 2.5, 7)
    for ang, ref in zip(r["det_angles"], r["det_rot"]):
        x, y, z = D.rotate_about_normal(dx, dy, dz, ang[0])
        x, y, z = D.rotate_about_vertical(x, y, z, ang[1])
        x, y, z = D.rotate_about_horizontal(x, y, z, ang[2])
        assert np.array_equal(np.stack([x, y, z]), ref)


def test_generate_detector_ints():
    v = golden("golden_voxel.npz")
    iq, qx, qy, qz = v["iq_plain"], v["qx"], v["qy"], v["qz"]
    x0, y0, z0, _, _ = O.init_detector(21, 1.2, (90.0, 30.0, 0.0),
                                       ("psi", "phi", "None"))
    shm = U.create_shared_array((21, 21))
    img = np.ndarray((21, 21), dtype=np.float64, buffer=shm.buf)
    img[:] = 0
    ref = np.zeros((21, 21))
    try:
        for ps, w in [(0.0, 0.25), (40.0, 0.5), (170.0, 0.25)]:
            D.generate_detector_ints((iq, qx, qy, qz, x0, y0, z0, ps, w, 12.0,
                                      1.0, 3.0, 1.0, shm.name))
            x, y, z = O.rotate_psi_phi_theta(x0, y0, z0, ps, 12.0, 3.0)
            ref += O.intersect_detector(iq, qx, qy, qz, x, y, z) * (w * 1.0 * 1.0)
        assert rel_l2(img.copy(), ref) <= 1e-15
    finally:
        del img
        shm.close()
        shm.unlink()


def test_generate_voxel_grid_low_mem(tmp_path):
    rng = np.random.default_rng(2)
    xyz, _ = W.graphite_slab((11.0, 10.0, 12.0), rng, disp_sigma=0.05)
    path = tmp_path / "slab.xyz"
    U.write_xyz(str(path), xyz, ["C"] * len(xyz))
    cx, _ = U.load_xyz(str(path))
    iq, qx, qy, qz = V.generate_voxel_grid_low_mem(str(path), 0.5, 0.2, 1.2, 1,
                                                   10000, "slab")
    ref = O.voxelgrid([(cx, np.full(len(cx), 6.0 + 0j))], 0.5, 0.2, 1.2, None,
                      False, 0, keep_full=True)
    full = np.divide(ref["full_sum"], ref["full_count"],
                     out=np.zeros_like(ref["full_sum"]),
                     where=ref["full_count"] != 0)
    assert np.array_equal(qx, ref["q"])
    assert rel_l2(iq, full) <= RTOL


def test_cli_main(tmp_path):
    """simulate_GIWAXS main() on a small graphite cell: slab, voxel grid,
    detector, positive-quadrant crop, saved outputs."""
    from giwaxsim_gb300 import simulate_GIWAXS as S
    cell = tmp_path / "cell.xyz"
    cxyz = np.array(W.GRAPHITE_BASIS) @ W.GRAPHITE_CELL
    U.write_xyz(str(cell), cxyz, ["C"] * len(cxyz))
    cfg = dict(input_filepath=str(cell), x_size="10", y_size="9", z_size="11",
               a="2.46", b="2.46", c="6.70", alpha="90", beta="90",
               gamma="120", r_voxel_size="0.5", q_voxel_size="0.2",
               max_q="1.2", energy="10000", fill_bkg="True", smooth="1",
               num_pixels="24", angle_init_val1="90", angle_init_ax1="psi",
               psi_start="0", psi_end="90", psi_num="7", phi_start="0",
               phi_end="0", phi_num="1", theta_start="0", theta_end="0",
               theta_num="1", mirror="True", save_folder=str(tmp_path / "out"))
    res = S.main(cfg)
    det, h, v = res["cell"]
    saved = np.load(tmp_path / "out" / "cell" / "det_sum.npy")
    assert np.array_equal(saved, det) and det.shape == (12, 12)
    assert (tmp_path / "out" / "cell" / "config.txt").exists()
    # the run's stage times
    import json
    m = json.load(open(tmp_path / "out" / "metrics.json"))
    names = [st["name"] for st in m["stages"]]
    assert names == ["slabs", "voxel", "detector", "save"]
    assert all(st["seconds"] >= 0 for st in m["stages"])
    assert m["total_seconds"] >= sum(st["seconds"] for st in m["stages"]) * 0.99
    assert m["device"]  # the GPU the run used
    # same pipeline through the oracle
    slab, el = S.slabmaker_fitting(str(cell), 10, 9, 11, 2.46, 2.46, 6.70, 90,
                                   90, 120)
    ref = O.voxelgrid([(slab, np.full(len(slab), 6.0 + 0j))], 0.5, 0.2, 1.2,
                      None, True, 1)
    rdet, rh, rv = O.detector(ref["iq"], ref["qx"], ref["qy"], ref["qz"], 24,
                              1.2, (90.0, 0.0, 0.0), ("psi", "None", "None"),
                              np.linspace(0, 90, 7), None, np.array([0.0]),
                              None, np.array([0.0]), None, mirror=True)
    kh, kv = np.where(rh >= 0)[0], np.where(rv >= 0)[0]
    assert rel_l2(det, rdet[np.ix_(kv, kh)]) <= RTOL
