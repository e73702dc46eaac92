"""Generate the golden fixtures in tests/golden/ by running the reference
GIWAXSim code itself (a Python package, imported from its checkout).

Run in a container that has the reference checkout, giving its path as the
first argument or in the environment variable GIWAXSIM_REFERENCE:
    python tests/golden/make_golden.py /path/to/reference
    python tests/golden/make_golden.py /path/to/reference pm6   # PM6 example
    (other fixture groups: slab, compare, multiq, shift)

The reference imports matplotlib, mpl_toolkits, fabio, lmfit and xraydb and
scipy.signal.tukey at module level; none of these is on the computation path
under test, so they are replaced with inert stubs and the tukey alias.  xraydb's
f'/f'' lookup returns 0, i.e. f = Z for every atom (the product and the oracle
take f values as an input, so this is the parity boundary).

Every fixture is small (the whole set is a few MB) so the CPU test suite loads
it in seconds.  Inputs are seeded and stored next to the outputs.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GIWAXSIM_REFERENCE")


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return lambda *a, **k: None


def _import_reference():
    if not REF or not os.path.isdir(REF):
        raise SystemExit("usage: make_golden.py /path/to/reference [group] "
                         "(or set GIWAXSIM_REFERENCE)")
    import scipy.signal
    import scipy.signal.windows
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.cm",
                 "matplotlib.ticker", "matplotlib.colors", "mpl_toolkits",
                 "mpl_toolkits.mplot3d", "xraydb", "fabio", "lmfit"]:
        m = _Stub(name)
        m.__path__ = []
        sys.modules[name] = m
    sys.modules["xraydb"].f1_chantler = lambda el, e: 0.0
    sys.modules["xraydb"].f2_chantler = lambda el, e: 0.0
    if not hasattr(scipy.signal, "tukey"):
        scipy.signal.tukey = scipy.signal.windows.tukey
    sys.path.insert(0, REF)
    from tools import comparison, detector, utilities, voxelgrids
    # The drivers accumulate into shared memory from a ThreadPoolExecutor;
    # concurrent np.add.at / += on the shared grids lose updates (on the PM6
    # example 340 of the 8.4 M cropped voxels differ between a threaded and
    # a serial run).  The fixtures run the reference's own drivers with a
    # single worker so that they are deterministic.
    import concurrent.futures as cf
    serial = lambda *a, **k: cf.ThreadPoolExecutor(max_workers=1)
    comparison.ThreadPoolExecutor = serial
    voxelgrids.ThreadPoolExecutor = serial
    return comparison, detector, utilities, voxelgrids


def small_graphite(seed=0, size=(12.0, 11.0, 13.0)):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from giwaxsim_gb300 import workloads
    rng = np.random.default_rng(seed)
    xyz, _ = workloads.graphite_slab(size, rng, disp_sigma=0.05)
    return xyz


def main():
    comparison, detector, utilities, voxelgrids = _import_reference()
    rng = np.random.default_rng(1234)

    # 1. rotations: atoms (np.dot(coords, R.T)) and detector planes
    #    (R @ vstack) -- pins the fused BLAS evaluation order.
    coords = rng.uniform(-60, 60, (300, 3))
    phis = np.concatenate([[0.0, 45.0, 90.0, 179.0],
                           rng.uniform(0, 180, 6)])
    rot = np.stack([utilities.rotate_coords_z(coords, p) for p in phis])
    dx, dy, dz, dh, dv = detector.make_detector(2.5, 9, 2.5, 7)
    det_rots = []
    angles = [(90.0, 30.0, 10.0), (12.5, 0.0, 0.0), (0.0, 47.0, 0.0),
              (0.0, 0.0, 33.0), (170.0, 95.0, 181.0)]
    for a in angles:
        x, y, z = detector.rotate_about_normal(dx, dy, dz, a[0])
        x, y, z = detector.rotate_about_vertical(x, y, z, a[1])
        x, y, z = detector.rotate_about_horizontal(x, y, z, a[2])
        det_rots.append(np.stack([x, y, z]))
    np.savez_compressed(os.path.join(HERE, "golden_rotation.npz"),
                        coords=coords, phis=phis, rot=rot,
                        det_angles=np.array(angles), det_rot=np.stack(det_rots))

    # 2. numpy floor division on values adjacent to multiples of the divisor
    bs = np.array([0.3, 0.25, 0.2, 0.03, 0.02, 0.015, 0.04095, 0.1])
    a_list, b_list = [], []
    for b in bs:
        k = rng.integers(-2000, 2000, 400).astype(np.float64)
        a = k * b
        for arr in (a, np.nextafter(a, np.inf), np.nextafter(a, -np.inf)):
            a_list.append(arr)
            b_list.append(np.full(arr.shape, b))
    fa, fb = np.concatenate(a_list), np.concatenate(b_list)
    np.savez_compressed(os.path.join(HERE, "golden_floordiv.npz"),
                        a=fa, b=fb, q=fa // fb)

    # 3. rectangular_collapse_lengths
    cases = []
    for phi in [0.0, 30.0, 45.0, 60.0, 89.0, 90.0, 91.0, 120.0, 135.0, 179.0,
                180.0] + list(rng.uniform(0, 180, 8)):
        for hor, ver in [(50.0, 50.0), (30.0, 70.0), (97.3, 41.2)]:
            xv = np.arange(350) * 0.3
            cases.append((phi, hor, ver,
                          voxelgrids.rectangular_collapse_lengths(
                              xv, hor, ver, phi).astype(np.float64)))
    np.savez_compressed(os.path.join(HERE, "golden_collapse.npz"),
                        phi=np.array([c[0] for c in cases]),
                        hor=np.array([c[1] for c in cases]),
                        ver=np.array([c[2] for c in cases]),
                        x=np.arange(350) * 0.3,
                        lengths=np.stack([c[3] for c in cases]))

    # 4. single slices through the reference's own per-slice worker
    #    (rotate_project_fft_coords -> process_file2), all fill/smooth modes.
    xyz = small_graphite(0)
    elements = np.array(["C"] * len(xyz))
    r, dq, max_q = 0.5, 0.15, 1.5
    g = int(np.ceil(2 * np.pi / (dq * r)))
    mqd = np.sqrt(2) * max_q
    mqd = mqd + mqd % dq
    qn = int((2 * mqd / dq) + 1)
    qn += (qn % 2 == 0)
    q = np.linspace(-mqd, mqd, qn)
    f_values = np.full(len(xyz), 6.0 + 0j)
    xb, yb, zb = [np.max(xyz[:, i]) - np.min(xyz[:, i]) for i in range(3)]
    avg = (np.sum(f_values) / (xb * yb * zb)) * r ** 3
    slice_phis = np.array([0.0, 17.0, 45.0, 90.0, 133.5])
    out = dict(coords=xyz, r=r, dq=dq, max_q=max_q, g=g, q=q,
               phis=slice_phis)
    for mode, (fill, smooth) in {"plain": (False, 0), "fill": (True, 0),
                                 "smooth": (False, 2),
                                 "fillsmooth": (True, 1)}.items():
        shm_s = utilities.create_shared_array((qn, qn, qn))
        shm_c = utilities.create_shared_array((qn, qn, qn))
        try:
            vs = np.ndarray((qn, qn, qn), dtype=np.float64, buffer=shm_s.buf)
            vc = np.ndarray((qn, qn, qn), dtype=np.float64, buffer=shm_c.buf)
            vs[:] = 0
            vc[:] = 0
            for phi in slice_phis:
                voxelgrids.rotate_project_fft_coords(
                    (xyz, f_values, phi, g, r, avg, xb, yb, zb, fill, smooth,
                     q, q, q, shm_s.name, shm_c.name))
            out["sum_" + mode] = vs.copy()
            out["count_" + mode] = vc.copy()
        finally:
            shm_s.close()
            shm_s.unlink()
            shm_c.close()
            shm_c.unlink()
    np.savez_compressed(os.path.join(HERE, "golden_slices.npz"), **out)

    # 5. the full voxel driver (automatic phis, threaded as shipped)
    xyz = small_graphite(1, size=(10.0, 10.0, 10.0))
    elements = np.array(["C"] * len(xyz))
    vox = {}
    for mode, (fill, smooth) in {"plain": (False, 0),
                                 "fillsmooth": (True, 1)}.items():
        iq, qx, qy, qz = comparison.voxelgridmaker_fitting(
            xyz, elements, 0.5, 0.2, 1.2, 10000, fill_bkg=fill, smooth=smooth)
        vox["iq_" + mode] = iq
    np.savez_compressed(os.path.join(HERE, "golden_voxel.npz"), coords=xyz,
                        r=0.5, dq=0.2, max_q=1.2, qx=qx, qy=qy, qz=qz, **vox)

    # 6. the detector driver on that grid (mirror=True: the shipped code
    #    reads a released buffer when mirror=False)
    iq = vox["iq_plain"]
    psis = np.linspace(0, 180, 7)
    dphis = np.array([0.0, 20.0])
    thetas = np.array([0.0, 5.0])
    det_sum, det_h, det_v = comparison.detectormaker_fitting(
        iq, qx, qy, qz, 21, 1.2, (90.0, 30.0, 10.0), ("psi", "phi", "theta"),
        psis, None, dphis, None, thetas, None, mirror=True)
    det_sum2, _, _ = comparison.detectormaker_fitting(
        iq, qx, qy, qz, 16, 1.2, (0.0, 0.0, 0.0), ("None", "None", "None"),
        np.linspace(0, 90, 10), None, np.array([0.0]), None,
        np.array([0.0]), None, mirror=True)
    # single orientations through generate_detector_ints' pieces
    x0, y0, z0, _, _ = detector.make_detector(1.2, 21, 1.2, 21)
    singles = []
    for a in [(0.0, 0.0, 0.0), (33.0, 12.0, 7.0), (90.0, 0.0, 0.0)]:
        x, y, z = detector.rotate_psi_phi_theta(x0, y0, z0, *a)
        singles.append(detector.intersect_detector(iq, qx, qy, qz, x, y, z))
    np.savez_compressed(os.path.join(HERE, "golden_detector.npz"),
                        det_sum=det_sum, det_h=det_h, det_v=det_v,
                        det_sum2=det_sum2, single_angles=np.array(
                            [(0.0, 0.0, 0.0), (33.0, 12.0, 7.0),
                             (90.0, 0.0, 0.0)]),
                        singles=np.stack(singles))
    # mirror fold on odd and even shapes
    mi = {}
    for shp in [(7, 9), (8, 6), (7, 6), (8, 9)]:
        a = rng.normal(size=shp)
        mi["in_%dx%d" % shp] = a
        mi["out_%dx%d" % shp] = detector.mirror_vertical_horizontal(a)
    np.savez_compressed(os.path.join(HERE, "golden_mirror.npz"), **mi)

    # 7. add_f0_q_3d and downselect_voxelgrid
    qa = np.linspace(-2.0, 2.0, 21)
    grid = rng.uniform(0, 1, (21, 21, 21))
    f0 = voxelgrids.add_f0_q_3d(grid, qa, qa, qa, "C")
    ds = voxelgrids.downselect_voxelgrid(grid, qa, qa, qa, 1.1)
    np.savez_compressed(os.path.join(HERE, "golden_f0.npz"), q=qa, grid=grid,
                        f0=f0, ds_grid=ds[0], ds_x=ds[1])
    print("fixtures written to", HERE)


def pm6():
    """The reference's shipped example (config_templates/
    simulate_GIWAXS_config.txt on test_input_files/PM6_sample.pdb): the unit
    cell, the reference's own result with f' = f'' = 0 (its shipped
    output_data/PM6_sample/det_sum.npy was made with xraydb's f', f'' at
    12.7 keV and a threaded run), and that shipped result.  Takes about six
    minutes (single-worker drivers)."""
    comparison, detector, utilities, voxelgrids = _import_reference()
    cfg = utilities.parse_config_file(
        os.path.join(REF, "config_templates", "simulate_GIWAXS_config.txt"))
    pdb = os.path.join(REF, "test_input_files", "PM6_sample.pdb")
    cell_xyz, cell_el = utilities.load_pdb(pdb)
    cell = utilities.load_pdb_cell_params(pdb)
    xs, ys, zs = (float(cfg[k]) for k in ("x_size", "y_size", "z_size"))
    slab, slab_el = comparison.slabmaker_fitting(pdb, xs, ys, zs, *cell)
    r, dq, mq = (float(cfg[k]) for k in ("r_voxel_size", "q_voxel_size", "max_q"))
    iq, qx, qy, qz = comparison.voxelgridmaker_fitting(
        slab, slab_el, r, dq, mq, float(cfg["energy"]), fill_bkg=True,
        smooth=int(cfg["smooth"]))
    psis = np.linspace(float(cfg["psi_start"]), float(cfg["psi_end"]),
                       int(cfg["psi_num"]))
    phis = np.linspace(float(cfg["phi_start"]), float(cfg["phi_end"]),
                       int(cfg["phi_num"]))
    thetas = np.linspace(float(cfg["theta_start"]), float(cfg["theta_end"]),
                         int(cfg["theta_num"]))
    init_vals = tuple(float(cfg[f"angle_init_val{i}"]) for i in (1, 2, 3))
    init_axs = tuple(cfg[f"angle_init_ax{i}"] for i in (1, 2, 3))
    det, h, v = comparison.detectormaker_fitting(
        iq, qx, qy, qz, int(cfg["num_pixels"]), mq, init_vals, init_axs, psis,
        None, phis, None, thetas, None, mirror=True)
    kh, kv = np.where(h >= 0)[0], np.where(v >= 0)[0]
    shipped = np.load(os.path.join(REF, "output_data", "PM6_sample",
                                   "det_sum.npy"))
    np.savez_compressed(
        os.path.join(HERE, "golden_pm6.npz"), cell_xyz=cell_xyz,
        cell_el=cell_el, cell=np.array(cell), slab_n=len(slab),
        slab_sum=slab.sum(0), slab_head=slab[:16], config=np.array(
            ["%s=%s" % kv_ for kv_ in cfg.items()]),
        det_ref=det[np.ix_(kv, kh)], det_h=h[kh], det_v=v[kv],
        det_shipped=shipped)
    print("PM6 fixture written")


SLAB_CASES = [
    # (name, cell source, cell parameters a b c alpha beta gamma, size)
    ("pm6", "pdb", None, (60.0, 40.0, 50.0)),
    ("graphite", "xyz", (2.46, 2.46, 6.70, 90.0, 90.0, 120.0), (20.0, 20.0, 20.0)),
    ("graphite_odd", "xyz", (2.46, 2.46, 6.70, 90.0, 90.0, 120.0), (33.3, 41.7, 25.0)),
    ("triclinic", "xyz", (4.1, 5.3, 6.2, 81.0, 95.0, 104.0), (27.5, 22.0, 31.0)),
]


def slab():
    """The reference's slabmaker_fitting (comparison.py:595-671) on the PM6
    cell and on small cells written as .xyz files (hexagonal graphite and a
    triclinic cell, so that b_x, c_x and c_y are not zero): atom count,
    a SHA-256 of the float64 coordinates and of the element names, and the
    first rows.  Seconds."""
    import hashlib
    import tempfile
    comparison, detector, utilities, voxelgrids = _import_reference()
    out = {}
    for name, kind, cellp, size in SLAB_CASES:
        if kind == "pdb":
            path = os.path.join(REF, "test_input_files", "PM6_sample.pdb")
            cellp = utilities.load_pdb_cell_params(path)
            cell_xyz, cell_el = utilities.load_pdb(path)
        else:
            av, bv, cv = utilities.calc_real_space_abc(*cellp)
            frac = np.array([[0, 0, 0.25], [0, 0, 0.75], [1 / 3, 2 / 3, 0.25],
                             [2 / 3, 1 / 3, 0.75], [0.1, 0.45, 0.6]])
            cell_xyz = frac @ np.array([av, bv, cv])
            cell_el = np.array(["C", "C", "C", "C", "S"])
            fd, path = tempfile.mkstemp(suffix=".xyz")
            with os.fdopen(fd, "w") as fh:
                fh.write("%d\ncell\n" % len(cell_xyz))
                for e, (x, y, z) in zip(cell_el, cell_xyz):
                    fh.write("%s %.17g %.17g %.17g\n" % (e, x, y, z))
            cell_xyz, cell_el = utilities.load_xyz(path)
        coords, els = comparison.slabmaker_fitting(path, *size, *cellp)
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        out[name + "_cell_xyz"] = cell_xyz
        out[name + "_cell_el"] = np.asarray(cell_el)
        out[name + "_cellp"] = np.array(cellp, dtype=np.float64)
        out[name + "_size"] = np.array(size)
        out[name + "_n"] = len(coords)
        out[name + "_sha"] = hashlib.sha256(coords.tobytes()).hexdigest()
        out[name + "_el_sha"] = hashlib.sha256(
            "".join(np.asarray(els).tolist()).encode()).hexdigest()
        out[name + "_head"] = coords[:8]
        if kind != "pdb":
            os.remove(path)
    np.savez_compressed(os.path.join(HERE, "golden_slab.npz"), **out)
    print("slab fixture written")


def compare():
    """The reference's experimental-comparison step on synthetic maps:
    trim_sim_data, rebin_qmap_and_mask (griddata, linear), the masking of
    fit_slabsize.py:142, optimize_scale_offset and the residual of
    fit_slabsize.py:43-44."""
    comparison, detector, utilities, voxelgrids = _import_reference()
    rng = np.random.default_rng(21)
    exp_qxy = np.linspace(0.05, 2.2, 97)
    exp_qz = np.linspace(0.02, 1.9, 83)
    gx, gz = np.meshgrid(exp_qxy, exp_qz)
    exp_img = (np.exp(-((np.hypot(gx, gz) - 1.4) / 0.08) ** 2) + 0.1 * gz
               + 0.02 * rng.random(gx.shape))
    mask = (rng.random(gx.shape) < 0.08).astype(int)
    mask[:, :4] = 1
    det_h = np.linspace(-2.5, 2.5, 120)
    det_v = np.linspace(-2.5, 2.5, 110)
    hx, vz = np.meshgrid(det_h, det_v)
    sim = (np.exp(-((np.hypot(hx, vz) - 1.38) / 0.09) ** 2) + 0.05
           + 0.01 * rng.random(hx.shape))
    sim_trim, h_trim, v_trim = comparison.trim_sim_data(sim, det_h, det_v,
                                                        exp_qxy, exp_qz)
    rebin_raw, rebin_mask = comparison.rebin_qmap_and_mask(
        h_trim, v_trim, exp_img, exp_qxy, exp_qz, mask)
    rebin_map = rebin_raw.copy()
    rebin_map[rebin_mask == 1] = 0
    scale, offset = comparison.optimize_scale_offset(sim_trim, rebin_map, rebin_mask)
    residual = (rebin_map - (scale * sim_trim + offset)) * (rebin_mask == 0)
    np.savez_compressed(
        os.path.join(HERE, "golden_compare.npz"), exp_qxy=exp_qxy,
        exp_qz=exp_qz, exp_img=exp_img, mask=mask, det_h=det_h, det_v=det_v,
        sim=sim, sim_trim=sim_trim, h_trim=h_trim, v_trim=v_trim,
        rebin_raw=rebin_raw, rebin_mask=rebin_mask, scale=scale,
        offset=offset, residual=residual)
    print("comparison fixture written")


MULTIQ_CASES = [
    # (name, fill_bkg, smooth, aff_num_qs)
    ("plain", False, 0, 3),
    ("fillsmooth", True, 1, 4),
]


def multiq():
    """The reference's generate_voxel_grid_low_mem (voxelgrids.py:535-722)
    with aff_num_qs > 1 on a small graphite slab in which every fifth atom is
    relabelled O (two elements, so the per-shell f values differ by more
    than a common factor), read back from an .xyz file.  f' = f'' = 0 (the
    xraydb stub), so f = f0(q_k).  Seconds."""
    import tempfile
    comparison, detector, utilities, voxelgrids = _import_reference()
    xyz = small_graphite(seed=5, size=(12.0, 11.0, 13.0))
    els = np.array(["O" if i % 5 == 0 else "C" for i in range(len(xyz))])
    fd, path = tempfile.mkstemp(suffix=".xyz")
    with os.fdopen(fd, "w") as fh:
        fh.write("%d\nslab\n" % len(xyz))
        for e, (x, y, z) in zip(els, xyz):
            fh.write("%s %.17g %.17g %.17g\n" % (e, x, y, z))
    coords, elements = utilities.load_xyz(path)
    r, dq, max_q = 0.5, 0.15, 1.0
    out = dict(coords=coords, elements=np.asarray(elements), r=r, dq=dq,
               max_q=max_q)
    for name, fill, smooth, K in MULTIQ_CASES:
        iq, qx, qy, qz = voxelgrids.generate_voxel_grid_low_mem(
            path, r, dq, max_q, K, 10000.0, "mq", output_dir=None,
            fill_bkg=fill, smooth=smooth)
        out[name + "_iq"] = iq
        out[name + "_K"] = K
        out[name + "_fill"] = fill
        out[name + "_smooth"] = smooth
        out["q"] = qx
    os.remove(path)
    np.savez_compressed(os.path.join(HERE, "golden_multiq.npz"), **out)
    print("multi-q fixture written")


SHIFT_CASES = [
    # (name, pad_width, pad_range (q))
    ("pad", 0.05, (1.2, 1.9)),
    ("nopad", 0.0, (1.2, 1.9)),
]


def shift():
    """The reference's shift_peak (comparison.py:566-592: linear_polar,
    add_pad, the zero mask, polar_linear) on a synthetic trimmed detector
    image with rings, on a positive-qxy grid like trim_sim_data leaves."""
    comparison, detector, utilities, voxelgrids = _import_reference()
    rng = np.random.default_rng(33)
    det_h = np.linspace(0.0, 2.4, 97)
    det_v = np.linspace(-0.1, 2.2, 83)
    hx, vz = np.meshgrid(det_h, det_v)
    q = np.hypot(hx, vz)
    img = (np.exp(-((q - 1.45) / 0.05) ** 2) + 0.5 * np.exp(-((q - 0.9) / 0.08) ** 2)
           + 0.05 + 0.01 * rng.random(q.shape))
    img[:3, :] = 0.0  # a zero band (the reference's mask keeps zeros zero)
    out = dict(det_h=det_h, det_v=det_v, img=img)
    for name, pw, pr in SHIFT_CASES:
        out[name + "_out"] = comparison.shift_peak(img.copy(), det_h, det_v, pw, pr)
        out[name + "_pw"] = pw
        out[name + "_pr"] = np.array(pr)
    np.savez_compressed(os.path.join(HERE, "golden_shift.npz"), **out)
    print("shift_peak fixture written")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "pm6":
        pm6()
    elif len(sys.argv) > 2 and sys.argv[2] == "slab":
        slab()
    elif len(sys.argv) > 2 and sys.argv[2] == "compare":
        compare()
    elif len(sys.argv) > 2 and sys.argv[2] == "multiq":
        multiq()
    elif len(sys.argv) > 2 and sys.argv[2] == "shift":
        shift()
    else:
        main()
