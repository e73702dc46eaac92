"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the GIWAXS forward path.

This module is the checker, not the product.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import it.  The
product (giwaxsim_gb300) never calls into it and fails loudly when its CUDA
library is missing.

It restates, in float64/complex128 numpy, the reference's forward path:

  tools/utilities.py:303-317   rotate_coords_z
  tools/voxelgrids.py:238-309  rectangular_collapse_lengths
  tools/voxelgrids.py:311-416  rotate_project_fft_coords  (deposit, fill_bkg,
                                smoothing, fftn/fftshift/|.|^2, slice axes)
  tools/voxelgrids.py:464-506  process_file2              (binning)
  tools/comparison.py:673-788  voxelgridmaker_fitting     (driver, divide,
                                crop, f0)
  tools/voxelgrids.py:16-48    downselect_voxelgrid
  tools/voxelgrids.py:828-857  add_f0_q_3d
  tools/detector.py:5-29       make_detector
  tools/detector.py:33-162     rotate_about_normal/horizontal/vertical
  tools/detector.py:194-232    intersect_detector (the second definition,
                                which shadows the first)
  tools/detector.py:234-244    rotate_psi_phi_theta
  tools/detector.py:246-275    mirror_vertical_horizontal
  tools/detector.py:278-300    generate_detector_ints
  tools/comparison.py:790-870  detectormaker_fitting
  old_modules/voxelgridmaker.py:56-61  averaging of I(q) over input files
  tools/comparison.py:595-671  slabmaker_fitting
  tools/comparison.py:469-592  linear_polar, polar_linear, add_pad, shift_peak
  tools/voxelgrids.py:535-722  generate_voxel_grid_low_mem, aff_num_qs > 1
  tools/utilities.py:318-340   get_element_f0_dict
  fit_slabsize.py:19-46        fullfit_model

Differences from the reference, all deliberate:
  * BLAS products are evaluated by oracle_fma.c as the explicit fused chain
    that OpenBLAS uses on x86_64 (pinned in tests/golden), so the oracle is
    bit-reproducible on any host.
  * phis may be passed explicitly (the reference always derives them).
  * the count grid is returned alongside I(q); accumulation is serial
    (voxelgrid_crop_threaded and detector_threaded spread slices and
    orientations over threads, with the additions guarded).
  * detectormaker copies the summed image before releasing it (the reference
    reads a closed shared-memory buffer when mirror=False).
  * smoothing accepts a non-integer sigma; mask edges are ceil(lo+sigma) and
    ceil(hi-sigma), which are the reference's slice bounds for integer sigma.

Parity status: pinned.  tests/golden holds outputs of the reference itself
(imported in a shim with f'=f''=0), and tests/test_oracle_golden.py checks this
module against them.  The xraydb f'/f'' lookup is not reproduced (xraydb is
not installed); f values are an input to both the oracle and the product.
"""
import ctypes
import math
import os
import threading

import numpy as np
from numpy.fft import fft2, fftshift
from scipy.ndimage import gaussian_filter1d, map_coordinates

_LIB = None
_LIB_LOCK = threading.Lock()


def _lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LIB_LOCK:
        return _load_lib()


def _load_lib():
    global _LIB
    if _LIB is None:
        from . import build_oracle
        path = build_oracle.build()
        lib = ctypes.CDLL(path)
        p = ctypes.c_void_p
        lib.oracle_rotate_rows.argtypes = [p, ctypes.c_int64, p, p]
        lib.oracle_rotate_rows.restype = None
        lib.oracle_rotate_xyz.argtypes = [p, p, p, ctypes.c_int64, p, p, p, p]
        lib.oracle_rotate_xyz.restype = None
        _LIB = lib
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fma_rows(pts, R):
    """np.dot(pts, R.T) with the BLAS fused evaluation order (n >= 2)."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    out = np.empty_like(pts)
    _lib().oracle_rotate_rows(_ptr(pts), len(pts), _ptr(R), _ptr(out))
    return out


def fma_xyz(x, y, z, R):
    """R @ vstack([x, y, z]) with the BLAS fused evaluation order."""
    shape = np.shape(x)
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    y = np.ascontiguousarray(y, dtype=np.float64).ravel()
    z = np.ascontiguousarray(z, dtype=np.float64).ravel()
    R = np.ascontiguousarray(R, dtype=np.float64)
    ox, oy, oz = np.empty_like(x), np.empty_like(y), np.empty_like(z)
    _lib().oracle_rotate_xyz(_ptr(x), _ptr(y), _ptr(z), len(x), _ptr(R),
                             _ptr(ox), _ptr(oy), _ptr(oz))
    return ox.reshape(shape), oy.reshape(shape), oz.reshape(shape)


# --------------------------------------------------------------------------
# tables: International Tables Vol. C, Table 6.1.1.4 (Cromer-Mann) for the
# elements the tests use, and atomic numbers.
Z_OF = {"H": 1, "C": 6, "N": 7, "O": 8, "F": 9, "Si": 14, "S": 16}
CROMER_MANN = {
    "C": (2.31, 20.8439, 1.02, 10.2075, 1.5886, 0.5687, 0.865, 51.6512, 0.2156),
    "H": (0.489918, 20.6593, 0.262003, 7.74039, 0.196767, 49.5519, 0.049879,
          2.20159, 0.001305),
    "N": (12.2126, 0.0057, 3.1322, 9.8933, 2.0125, 28.9975, 1.1663, 0.5826,
          -11.529),
    "O": (3.0485, 13.2771, 2.2868, 5.7011, 1.5463, 0.3239, 0.867, 32.9089,
          0.2508),
    "F": (3.5392, 10.2825, 2.6412, 4.2944, 1.517, 0.2615, 1.0243, 26.1476,
          0.2776),
    "Si": (6.2915, 2.4386, 3.0353, 32.3337, 1.9891, 0.6785, 1.541, 81.6937,
           1.1407),
    "S": (6.9053, 1.4679, 5.2034, 22.2151, 1.4379, 0.2536, 1.5863, 56.172,
          0.8669),
}


# --------------------------------------------------------------------------
# voxel path

def rotate_coords_z(coords, phi):
    """utilities.py:303-317: coords @ Rz(phi).T."""
    pr = np.radians(phi)
    R = np.array([[np.cos(pr), -np.sin(pr), 0],
                  [np.sin(pr), np.cos(pr), 0],
                  [0, 0, 1]])
    return fma_rows(coords, R)


def rectangular_collapse_lengths(x_vals, hor_length, ver_length, phi):
    """voxelgrids.py:238-309, vectorised with the same branch order and the
    same floating-point expression trees."""
    x_vals = np.asarray(x_vals, dtype=np.float64)
    if phi > 90:
        phi = phi - 90
        hor_length, ver_length = ver_length, hor_length
    theta = 90 - phi
    theta_rad = np.deg2rad(theta)
    phi_rad = np.deg2rad(phi)
    if phi == 0:
        return np.where(x_vals < hor_length, ver_length, 0).astype(np.float64)
    if phi == 90:
        return np.where(x_vals < ver_length, hor_length, 0).astype(np.float64)
    stop1 = ver_length * np.cos(theta_rad)
    stop2 = hor_length * np.cos(phi_rad)
    if stop1 < stop2:
        mid_length = ver_length / np.sin(theta_rad)
    else:
        stop1, stop2 = stop2, stop1
        mid_length = hor_length / np.sin(phi_rad)
    out = np.zeros_like(x_vals)
    vc = ver_length * np.cos(theta_rad)
    base = np.sqrt(ver_length ** 2 - vc ** 2)
    tphi = np.tan(phi_rad)
    ttheta = np.tan(theta_rad)
    cphi = np.cos(phi_rad)
    ctheta = np.cos(theta_rad)
    for i, x in enumerate(x_vals):
        if x == 0:
            v = 0.0
        elif x < stop1:
            v = (base + x * tphi) - ((vc - x) * ttheta)
        elif x <= stop2:
            v = mid_length
        elif x < stop1 + stop2:
            v = (hor_length - ((x - vc) / cphi)) / ctheta
        else:
            v = 0.0
        out[i] = v
    return out


def mask_bounds(lo, hi, sigma, n):
    """Start/stop of the smoothing plateau mask[lo+sigma : hi-sigma] with
    Python slice normalisation (voxelgrids.py:369-370); ceil() extends the
    bounds to non-integer sigma."""
    start = int(math.ceil(lo + sigma))
    stop = int(math.ceil(hi - sigma))
    s, e, _ = slice(start, stop).indices(n)
    return s, e


def smooth_profile(n, lo, hi, sigma):
    """gaussian_filter1d(mask, sigma, mode='wrap') of the plateau mask."""
    m = np.zeros(n)
    s, e = mask_bounds(lo, hi, sigma, n)
    m[s:e] = 1
    return gaussian_filter1d(m, sigma=sigma, mode="wrap")


def project_slice(coords, f_values, phi, grid_size, r_voxel_size, avg_voxel_f,
                  x_bound, y_bound, z_bound, fill_bkg, smooth):
    """voxelgrids.py:318-379: rotate, shift, nearest-bin deposit, fill, smooth.
    Returns (grid complex128 (g,g) [z,y], info dict)."""
    g = grid_size
    rot = rotate_coords_z(coords, phi)
    rot[:, 0] -= np.min(rot[:, 0])
    rot[:, 1] -= np.min(rot[:, 1])
    rot[:, 2] -= np.min(rot[:, 2])
    yi = (rot[:, 1] // r_voxel_size).astype(int)
    zi = (rot[:, 2] // r_voxel_size).astype(int)
    ok = (yi >= 0) & (yi < g) & (zi >= 0) & (zi < g)
    yi, zi, fv = yi[ok], zi[ok], f_values[ok]
    grid = np.zeros((g, g), dtype=complex)
    np.add.at(grid, (zi, yi), fv)
    max_voxels = np.sqrt(x_bound ** 2 + y_bound ** 2) // r_voxel_size
    y_min, z_min = np.min(yi), np.min(zi)
    y_max, z_max = np.max(yi), np.max(zi)
    if fill_bkg:
        xv = np.arange(g) * r_voxel_size
        lengths = rectangular_collapse_lengths(xv, y_bound, x_bound, phi)
        missing = (max_voxels - (lengths // r_voxel_size)).astype(int)
        grid = grid + np.tile(missing * avg_voxel_f, (g, 1))
        fillv = avg_voxel_f * max_voxels
        grid[:z_min, :] = fillv
        grid[z_max:, :] = fillv
        grid[z_min:z_max + 1, :y_min + 1] = fillv
        grid[z_min:z_max + 1, y_max:] = fillv
    if smooth:
        avg_val = avg_voxel_f * max_voxels
        my = smooth_profile(g, y_min, y_max, smooth)
        mz = smooth_profile(g, z_min, z_max, smooth)
        M = np.outer(mz, my)
        grid = grid * M + avg_val * (1 - M)
    info = dict(y_idx=yi, z_idx=zi, valid=ok, y_min=y_min, y_max=y_max,
                z_min=z_min, z_max=z_max, max_voxels=max_voxels)
    return grid, info


def slice_intensity(grid):
    """voxelgrids.py:388-392: |fftshift(fftn(grid))|^2."""
    return np.abs(fftshift(fft2(grid))) ** 2


def slice_axes(grid_size, r_voxel_size, phi):
    """voxelgrids.py:382-402: (det_h_qx, det_h_qy, det_v_qz)."""
    q_h = fftshift(np.fft.fftfreq(grid_size, d=r_voxel_size) * 2 * np.pi)
    q_v = fftshift(np.fft.fftfreq(grid_size, d=r_voxel_size) * 2 * np.pi)
    right_qy = np.max(q_h) * np.cos(np.deg2rad(-phi))
    right_qx = -np.max(q_h) * np.sin(np.deg2rad(-phi))
    hy = np.linspace(-right_qy, right_qy, num=len(q_h))
    hx = np.linspace(-right_qx, right_qx, num=len(q_h))
    return hx, hy, q_v


def bin_indices(det_h_qx, det_h_qy, det_v_qz, qx, qy, qz):
    """voxelgrids.py:474-499: masks and flat voxel indices of one slice.
    Returns (v_mask, h_mask, qy_idx[h], qx_idx[h], qz_idx[v])."""
    hm = ((det_h_qx <= np.max(qx)) & (det_h_qx >= np.min(qx))
          & (det_h_qy <= np.max(qy)) & (det_h_qy >= np.min(qy)))
    vm = (det_v_qz <= np.max(qz)) & (det_v_qz >= np.min(qz))
    dq = np.diff(qz)[0]
    ix = ((det_h_qx[hm] - np.min(qx)) // dq).astype(int)
    iy = ((det_h_qy[hm] - np.min(qy)) // dq).astype(int)
    iz = ((det_v_qz[vm] - np.min(qz)) // dq).astype(int)
    return vm, hm, iy, ix, iz


def crop_pairs(iq_2d, det_h_qx, det_h_qy, det_v_qz, q, lo, Qc):
    """The pixels of one slice that process_file2 (voxelgrids.py:464-506)
    bins into the cropped cube q[lo:lo+Qc]^3, as flat crop indices
    ((iy*Qc + ix)*Qc + iz) and intensities."""
    vm, hm, iy, ix, iz = bin_indices(det_h_qx, det_h_qy, det_v_qz, q, q, q)
    ky, kx, kz = iy - lo, ix - lo, iz - lo
    oh = (ky >= 0) & (ky < Qc) & (kx >= 0) & (kx < Qc)
    ov = (kz >= 0) & (kz < Qc)
    sub = iq_2d[vm, :][:, hm][ov, :][:, oh]
    flat = (ky[oh] * Qc + kx[oh])[None, :] * Qc + kz[ov][:, None]
    return flat.ravel().astype(np.int64), sub.ravel()


def crop_window(q, max_q):
    """First index and length of downselect_voxelgrid's crop of axis q."""
    idx = np.where(np.abs(q) < max_q + np.abs(q[1] - q[0]))[0]
    return int(idx[0]), int(idx[-1] - idx[0] + 1)


def bin_slice(iq_2d, det_h_qx, det_h_qy, det_v_qz, qx, qy, qz, vsum, vcount):
    """voxelgrids.py:464-506 (process_file2) into plain arrays."""
    vm, hm, iy, ix, iz = bin_indices(det_h_qx, det_h_qy, det_v_qz, qx, qy, qz)
    sub = iq_2d[vm, :][:, hm]
    IY = np.broadcast_to(iy[None, :], sub.shape).ravel()
    IX = np.broadcast_to(ix[None, :], sub.shape).ravel()
    IZ = np.broadcast_to(iz[:, None], sub.shape).ravel()
    np.add.at(vsum, (IY, IX, IZ), sub.ravel())
    np.add.at(vcount, (IY, IX, IZ), 1.0)


def voxel_geometry(r_voxel_size, q_voxel_size, max_q, coords=None):
    """comparison.py:704-731: checks, grid size, q axis, automatic phis."""
    max_q_diag = np.sqrt(2) * max_q
    if max_q_diag > 2 * np.pi / r_voxel_size:
        raise Exception("Max_q is non-physical for given voxel size")
    grid_size = int(np.ceil(2 * np.pi / (q_voxel_size * r_voxel_size)))
    if coords is not None:
        b = [np.max(coords[:, i]) - np.min(coords[:, i]) for i in range(3)]
        if grid_size * r_voxel_size < np.min(b):
            raise Exception("Calculated real-space bounds smaller than "
                            "simulation. Please lower delta_q value")
    max_q_diag = max_q_diag + max_q_diag % q_voxel_size
    q_num = ((2 * max_q_diag / q_voxel_size) + 1).astype(int)
    if q_num % 2 == 0:
        q_num += 1
    q = np.linspace(-max_q_diag, max_q_diag, q_num)
    dphi = np.arctan(q_voxel_size / max_q_diag)
    phi_num = np.ceil(2 * np.pi / dphi).astype(int)
    phis = np.linspace(0, 180 - (180 / phi_num), num=phi_num)
    return grid_size, q, phis


def downselect_voxelgrid(grid, x_axis, y_axis, z_axis, max_val):
    """voxelgrids.py:16-48."""
    vs = np.abs(x_axis[1] - x_axis[0])
    max_val = max_val + vs
    xi = np.where(np.abs(x_axis) < max_val)[0]
    yi = np.where(np.abs(y_axis) < max_val)[0]
    zi = np.where(np.abs(z_axis) < max_val)[0]
    sub = grid[yi[0]:yi[-1] + 1, xi[0]:xi[-1] + 1, zi[0]:zi[-1] + 1]
    return (sub, x_axis[xi[0]:xi[-1] + 1], y_axis[yi[0]:yi[-1] + 1],
            z_axis[zi[0]:zi[-1] + 1])


def f0_factor(qx_axis, qy_axis, qz_axis, element="C"):
    """voxelgrids.py:838-854: ((sum_i a_i exp(-b_i q^2/16pi^2) + c)/Z)^2."""
    Z = Z_OF[element]
    a = CROMER_MANN[element]
    qx, qy, qz = np.meshgrid(qx_axis, qy_axis, qz_axis)
    q2 = qx ** 2 + qy ** 2 + qz ** 2
    s = 16 * np.pi ** 2
    return ((a[0] * np.exp(-a[1] * q2 / s) + a[2] * np.exp(-a[3] * q2 / s)
             + a[4] * np.exp(-a[5] * q2 / s) + a[6] * np.exp(-a[7] * q2 / s)
             + a[8]) / Z) ** 2


def add_f0_q_3d(iq, qx_axis, qy_axis, qz_axis, element="C"):
    """voxelgrids.py:828-857."""
    return iq * f0_factor(qx_axis, qy_axis, qz_axis, element)


def structure_constants(coords, f_values, r_voxel_size):
    """comparison.py:712-744: bounds and the average voxel scattering factor."""
    xb = np.max(coords[:, 0]) - np.min(coords[:, 0])
    yb = np.max(coords[:, 1]) - np.min(coords[:, 1])
    zb = np.max(coords[:, 2]) - np.min(coords[:, 2])
    avg = (np.sum(f_values) / (xb * yb * zb)) * r_voxel_size ** 3
    return xb, yb, zb, avg


def voxelgrid(structures, r_voxel_size, q_voxel_size, max_q, phis=None,
              fill_bkg=False, smooth=0, f0_element="C", keep_full=False):
    """comparison.py:673-788 restated; `structures` is a list of
    (coords (N,3) float64, f_values (N,) complex128).  With several
    structures the cropped I(q) grids are averaged before the f0 factor, as
    old_modules/voxelgridmaker.py:56-72 does.

    Returns dict(iq, qx, qy, qz, count, sum) -- count/sum are the cropped
    count and sum grids of the last structure's accumulation (counts are
    structure independent)."""
    grid_size, q, auto_phis = voxel_geometry(r_voxel_size, q_voxel_size, max_q,
                                             structures[0][0])
    if phis is None:
        phis = auto_phis
    qn = len(q)
    iq_acc = None
    for coords, fv in structures:
        voxel_geometry(r_voxel_size, q_voxel_size, max_q, coords)
        xb, yb, zb, avg = structure_constants(coords, fv, r_voxel_size)
        vsum = np.zeros((qn, qn, qn))
        vcnt = np.zeros((qn, qn, qn))
        for phi in phis:
            grid, _ = project_slice(coords, fv, phi, grid_size, r_voxel_size,
                                    avg, xb, yb, zb, fill_bkg, smooth)
            iq2 = slice_intensity(grid)
            hx, hy, vz = slice_axes(grid_size, r_voxel_size, phi)
            bin_slice(iq2, hx, hy, vz, q, q, q, vsum, vcnt)
        iq = np.divide(vsum, vcnt, out=np.zeros_like(vsum), where=vcnt != 0)
        iq_s, qxs, qys, qzs = downselect_voxelgrid(iq, q, q, q, max_q)
        iq_acc = iq_s.copy() if iq_acc is None else iq_acc + iq_s
    iq_acc = iq_acc / len(structures) if len(structures) > 1 else iq_acc
    out = dict(iq=add_f0_q_3d(iq_acc, qxs, qys, qzs, f0_element),
               qx=qxs, qy=qys, qz=qzs,
               count=downselect_voxelgrid(vcnt, q, q, q, max_q)[0],
               sum=downselect_voxelgrid(vsum, q, q, q, max_q)[0],
               grid_size=grid_size, q=q, phis=np.asarray(phis))
    if keep_full:
        out["full_sum"], out["full_count"] = vsum, vcnt
    return out


def _crop_chunk(payload):
    (coords, fv, phis, g, r, fill, smooth, q, consts, lo, Qc, vsum, vcnt,
     lock) = payload
    xb, yb, zb, avg = consts
    for phi in phis:
        grid, _ = project_slice(coords, fv, phi, g, r, avg, xb, yb, zb, fill,
                                smooth)
        hx, hy, vz = slice_axes(g, r, phi)
        i, v = crop_pairs(slice_intensity(grid), hx, hy, vz, q, lo, Qc)
        with lock:  # process_file2's np.add.at, one slice at a time
            np.add.at(vsum, i, v)
            np.add.at(vcnt, i, 1.0)


def voxelgrid_crop_threaded(coords, f_values, r_voxel_size, q_voxel_size,
                            max_q, phis, fill_bkg=False, smooth=0, workers=8):
    """voxelgrid() for one structure, with the slices spread over `workers`
    threads as the reference's driver does (comparison.py:759-763) and only
    the cropped cube accumulated (downselect_voxelgrid keeps nothing else).
    Threads add their slices into one shared pair of grids under a lock:
    the reference's unguarded np.add.at from threads loses updates.  Sums
    are added in another order than the serial voxelgrid() (differences at
    the float64 rounding level); counts are identical.
    Returns dict(iq, count, q) over the crop."""
    from concurrent.futures import ThreadPoolExecutor
    grid_size, q, _ = voxel_geometry(r_voxel_size, q_voxel_size, max_q, coords)
    lo, Qc = crop_window(q, max_q)
    phis = np.asarray(phis)
    chunks = [c for c in (phis[i::workers] for i in range(workers)) if len(c)]
    consts = structure_constants(coords, f_values, r_voxel_size)
    vsum = np.zeros(Qc ** 3)
    vcnt = np.zeros(Qc ** 3)
    lock = threading.Lock()
    _lib()  # build/load the helper before the threads use it
    with ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(_crop_chunk, [
            (coords, f_values, c, grid_size, r_voxel_size, fill_bkg, smooth,
             q, consts, lo, Qc, vsum, vcnt, lock) for c in chunks]))
    iq = np.divide(vsum, vcnt, out=np.zeros_like(vsum), where=vcnt != 0)
    qc = q[lo:lo + Qc]
    iq = add_f0_q_3d(iq.reshape(Qc, Qc, Qc), qc, qc, qc, "C")
    return dict(iq=iq, count=vcnt.reshape(Qc, Qc, Qc), q=qc)


# --------------------------------------------------------------------------
# shift_peak (comparison.py:469-592): polar warp, pi-pi peak padding, back

def to_polar(img, centre, radius):
    """comparison.py:469-499 (linear_polar, order 1, cval 0) with the output
    shape (round(2 pi radius), round(radius))."""
    n_t, n_r = int(round(radius * 2 * np.pi)), int(round(radius))
    rr = np.linspace(0, radius, n_r)
    tt = np.linspace(0, 2 * np.pi, n_t)
    cols = rr * np.cos(tt[:, None]) + centre[1]
    rows = rr * np.sin(tt[:, None]) + centre[0]
    out = np.zeros((n_t, n_r), dtype=img.dtype)
    map_coordinates(img, (rows, cols), order=1, output=out, cval=0)
    return out


def from_polar(polar, centre, shape):
    """comparison.py:501-538 (polar_linear, r = polar width, order 1)."""
    n_t, n_r = polar.shape
    o = np.array(centre)
    yy, xx = np.mgrid[:shape[0], :shape[1]] - o[:, None, None]
    rad = np.sqrt(yy ** 2 + xx ** 2)
    ang = np.arctan2(yy, xx)
    ang[ang < 0] += 2 * np.pi
    rad = (rad / n_r) * (n_r - 1)
    ang = (ang / (2 * np.pi)) * (n_t - 1)
    out = np.zeros(shape, dtype=polar.dtype)
    map_coordinates(polar, (ang, rad), order=1, output=out, cval=0)
    return out


def pad_columns(polar, r_axis, pad_width, pad_range):
    """comparison.py:540-563 (add_pad): duplicate round(pad_width/pixel)
    columns evenly spread from pad_range[0] on, then drop as many columns at
    the far end."""
    steps = np.diff(r_axis)
    px = np.mean(steps[steps > 0])
    n_pad = int(np.round(pad_width / px))
    if n_pad == 0:
        return polar
    i0 = int(np.argmin(np.abs(r_axis - pad_range[0])))
    i1 = int(np.argmin(np.abs(r_axis - pad_range[1])))
    gap = int((i1 - i0 - 1) / n_pad - 1)
    assert gap >= 0, "pad_range is too small for desired pad_width"
    for k in range(n_pad):
        at = i0 + 2 * k + gap * k
        polar = np.insert(polar, at + 1, polar[:, at], axis=1)
    return polar[:, :-n_pad]


def shift_peak(image, det_h, det_v, pad_width, pad_range):
    """comparison.py:566-592."""
    hh, vv = np.meshgrid(det_h, det_v)
    qr = np.hypot(hh, vv)
    radius = float(np.sqrt(image.shape[0] ** 2 + image.shape[1] ** 2))
    centre = (int(np.argmin(np.abs(det_v))), int(np.argmin(np.abs(det_h))))
    polar = to_polar(image, centre, radius)
    r_axis = to_polar(qr, centre, radius)[0, :]
    padded = pad_columns(polar.copy(), r_axis, pad_width, pad_range)
    padded[polar == 0] = 0
    return from_polar(padded, centre, image.shape)


# --------------------------------------------------------------------------
# multi-q form factors (generate_voxel_grid_low_mem with aff_num_qs > 1)

def element_f0_at(q_val, element):
    """utilities.py:318-340 get_element_f0_dict for one element: the
    Cromer-Mann sum with exponent -b q/(16 pi^2) (q, not q^2, as the
    reference writes it)."""
    a = CROMER_MANN[element]
    s = 16 * np.pi ** 2
    return (a[0] * np.exp(-a[1] * q_val / s) + a[2] * np.exp(-a[3] * q_val / s)
            + a[4] * np.exp(-a[5] * q_val / s) + a[6] * np.exp(-a[7] * q_val / s)
            + a[8])


def aff_shells(max_q_diag, aff_num_qs):
    """voxelgrids.py:659-664: shell centres and (lower, upper] bounds."""
    K = int(aff_num_qs)
    step = max_q_diag / K
    q_vals = np.array([0.5 * step + k * step for k in range(K)])
    return q_vals, q_vals - step / 2, q_vals + step / 2


def shell_masks(q, lower, upper):
    """voxelgrids.py:651-652, :706: (qr <= upper) & (qr > lower) per shell on
    the meshgrid |q| of the full axis."""
    qx, qy, qz = np.meshgrid(q, q, q)
    qr = np.sqrt(qx ** 2 + qy ** 2 + qz ** 2)
    return [(qr <= u) & (qr > l) for l, u in zip(lower, upper)]


def voxelgrid_multi_q(coords, elements, f1f2, r_voxel_size, q_voxel_size,
                      max_q, aff_num_qs, phis=None, fill_bkg=False, smooth=0,
                      mode="reference"):
    """voxelgrids.py:535-722 with aff_num_qs > 1 on the full q grid.  f1f2:
    element -> f' + i f''.  Per shell k the atoms scatter with f0(q_k) + f'
    + i f'' (no Z: the reference's multi-q branch, :665-669) and the average
    voxel f follows (:671-674).

    mode "reference": what the reference returns.  Its loop overwrites the
    grid with each shell's I(q) and then adds the shell-masked grid to
    itself (:703-707), so the result is the last shell's I(q) with the last
    shell doubled.
    mode "per_shell": the evident intent, sum over k of shell k's I(q) masked
    to shell k.

    Returns dict(iq, q, masks, shell_iq) with shell_iq the per-shell grids."""
    grid_size, q, auto_phis = voxel_geometry(r_voxel_size, q_voxel_size, max_q,
                                             coords)
    if phis is None:
        phis = auto_phis
    q_vals, lower, upper = aff_shells(q[-1], aff_num_qs)
    masks = shell_masks(q, lower, upper)
    elements = np.asarray(elements)
    qn = len(q)
    shells = range(len(q_vals)) if mode == "per_shell" else [len(q_vals) - 1]
    shell_iq = {}
    for k in shells:
        fv = np.array([element_f0_at(q_vals[k], e) + f1f2[e] for e in elements],
                      dtype=complex)
        xb, yb, zb, avg = structure_constants(coords, fv, r_voxel_size)
        vsum = np.zeros((qn, qn, qn))
        vcnt = np.zeros((qn, qn, qn))
        for phi in phis:
            grid, _ = project_slice(coords, fv, phi, grid_size, r_voxel_size,
                                    avg, xb, yb, zb, fill_bkg, smooth)
            hx, hy, vz = slice_axes(grid_size, r_voxel_size, phi)
            bin_slice(slice_intensity(grid), hx, hy, vz, q, q, q, vsum, vcnt)
        shell_iq[k] = np.divide(vsum, vcnt, out=np.zeros_like(vsum),
                                where=vcnt != 0)
    if mode == "per_shell":
        iq = np.zeros((qn, qn, qn))
        for k, m in enumerate(masks):
            iq += np.where(m, shell_iq[k], 0)
    else:
        last = shell_iq[len(q_vals) - 1]
        iq = last + np.where(masks[-1], last, 0)
    return dict(iq=iq, q=q, masks=masks, shell_iq=shell_iq, lower=lower,
                upper=upper, q_vals=q_vals, phis=np.asarray(phis))


# --------------------------------------------------------------------------
# detector path

def rotation_matrix(u, theta):
    """utilities.py:222-245 (Rodrigues), same expression trees."""
    ux, uy, uz = u[0], u[1], u[2]
    R = np.zeros((3, 3))
    c, s = np.cos(theta), np.sin(theta)
    R[0, 0] = c + ux ** 2 * (1 - c)
    R[0, 1] = ux * uy * (1 - c) - uz * s
    R[0, 2] = ux * uz * (1 - c) + uy * s
    R[1, 0] = uy * ux * (1 - c) + uz * s
    R[1, 1] = c + uy ** 2 * (1 - c)
    R[1, 2] = uy * uz * (1 - c) - ux * s
    R[2, 0] = uz * ux * (1 - c) - uy * s
    R[2, 1] = uz * uy * (1 - c) + ux * s
    R[2, 2] = c + uz ** 2 * (1 - c)
    return R


def make_detector(h_max, nh, v_max, nv):
    """detector.py:5-29."""
    h = np.linspace(-h_max, h_max, nh)
    v = np.linspace(-v_max, v_max, nv)
    y, z = np.meshgrid(h, v)
    return np.zeros_like(y), y, z, h, v


def _corner(x, y, z, i, j):
    return np.array([x[i, j], y[i, j], z[i, j]])


def axis_matrix(x, y, z, kind, angle_deg):
    """The rotation matrix each of detector.py:33-162 builds from the current
    grid's corners."""
    p1 = _corner(x, y, z, 0, 0)
    if kind == "psi":
        v1 = _corner(x, y, z, 0, -1) - p1
        v2 = _corner(x, y, z, -1, 0) - p1
        ax = np.cross(v1, v2)
    elif kind == "theta":
        ax = _corner(x, y, z, 0, -1) - p1
    elif kind == "phi":
        ax = _corner(x, y, z, -1, 0) - p1
    else:
        raise ValueError(kind)
    ax = ax / np.linalg.norm(ax)
    return rotation_matrix(ax, np.radians(angle_deg))


def rotate_about(x, y, z, kind, angle_deg):
    R = axis_matrix(x, y, z, kind, angle_deg)
    return fma_xyz(x, y, z, R)


def rotate_psi_phi_theta(x, y, z, psi, phi, theta):
    """detector.py:234-244."""
    x, y, z = rotate_about(x, y, z, "psi", psi)
    x, y, z = rotate_about(x, y, z, "phi", phi)
    x, y, z = rotate_about(x, y, z, "theta", theta)
    return x, y, z


def intersect_indices(iq_shape, qx, qy, qz, x, y, z):
    """detector.py:213-224: clipped voxel indices of each pixel."""
    dq = np.diff(qz)[0]
    ix = ((x.ravel() - np.min(qx)) // dq).astype(int)
    iy = ((y.ravel() - np.min(qy)) // dq).astype(int)
    iz = ((z.ravel() - np.min(qz)) // dq).astype(int)
    ix = np.clip(ix, 0, iq_shape[1] - 1)
    iy = np.clip(iy, 0, iq_shape[0] - 1)
    iz = np.clip(iz, 0, iq_shape[2] - 1)
    return iy, ix, iz


def intersect_detector(iq, qx, qy, qz, x, y, z):
    """detector.py:194-232."""
    iy, ix, iz = intersect_indices(iq.shape, qx, qy, qz, x, y, z)
    return iq[iy, ix, iz].reshape(x.shape)


def mirror_vertical_horizontal(qmap):
    """detector.py:246-275."""
    lr = np.fliplr(qmap)
    ud = np.flipud(qmap)
    udlr = np.fliplr(ud)
    out = qmap + lr + ud + udlr
    nr, nc = qmap.shape
    if nr % 2:
        row = qmap[nr // 2, :]
        out[nr // 2, :] = (row + row[::-1]) * 2
    if nc % 2:
        col = qmap[:, nc // 2]
        out[:, nc // 2] = (col + col[::-1]) * 2
    if nr % 2 and nc % 2:
        out[nr // 2, nc // 2] = qmap[nr // 2, nc // 2] * 4
    return out


def init_detector(num_pixels, max_q, angle_init_vals, angle_init_axs):
    """comparison.py:792-818."""
    x, y, z, h, v = make_detector(max_q, num_pixels, max_q, num_pixels)
    for val, ax in zip(angle_init_vals, angle_init_axs):
        if ax in ("psi", "phi", "theta"):
            x, y, z = rotate_about(x, y, z, ax, val)
    return x, y, z, h, v


def orientation_list(psis, psi_w, phis, phi_w, thetas, theta_w):
    """comparison.py:836-841 ordering: psi outer, phi, theta inner."""
    out = []
    for ps, pw in zip(psis, psi_w):
        for ph, hw in zip(phis, phi_w):
            for th, tw in zip(thetas, theta_w):
                out.append((ps, pw, ph, hw, th, tw))
    return out


def detector(iq, qx, qy, qz, num_pixels, max_q, angle_init_vals,
             angle_init_axs, psis, psi_weights, phis, phi_weights, thetas,
             theta_weights, mirror=True):
    """comparison.py:790-870 restated with weights passed as arrays (None ->
    uniform) and a serial orientation loop."""
    x0, y0, z0, h, v = init_detector(num_pixels, max_q, angle_init_vals,
                                     angle_init_axs)
    psis, phis, thetas = map(np.asarray, (psis, phis, thetas))
    psi_weights = (np.ones_like(psis) / len(psis) if psi_weights is None
                   else np.asarray(psi_weights))
    phi_weights = (np.ones_like(phis) / len(phis) if phi_weights is None
                   else np.asarray(phi_weights))
    theta_weights = (np.ones_like(thetas) / len(thetas) if theta_weights is None
                     else np.asarray(theta_weights))
    acc = detector_partial(iq, qx, qy, qz, x0, y0, z0, orientation_list(
        psis, psi_weights, phis, phi_weights, thetas, theta_weights))
    return detector_epilogue(acc, mirror), h, v


def detector_threaded(iq, qx, qy, qz, num_pixels, max_q, angle_init_vals,
                      angle_init_axs, psis, psi_weights, phis, phi_weights,
                      thetas, theta_weights, mirror=True, workers=8):
    """detector() with the orientation list split over `workers` threads
    (the reference's driver sums orientations from a thread pool,
    comparison.py:850-853); the partial images are added at the end."""
    from concurrent.futures import ThreadPoolExecutor
    x0, y0, z0, h, v = init_detector(num_pixels, max_q, angle_init_vals,
                                     angle_init_axs)
    psis, phis, thetas = map(np.asarray, (psis, phis, thetas))
    w = [np.ones_like(a) / len(a) if wa is None else np.asarray(wa)
         for a, wa in ((psis, psi_weights), (phis, phi_weights),
                       (thetas, theta_weights))]
    orients = orientation_list(psis, w[0], phis, w[1], thetas, w[2])
    chunks = [c for c in (orients[i::workers] for i in range(workers)) if c]
    _lib()
    with ThreadPoolExecutor(max_workers=workers) as ex:
        parts = list(ex.map(lambda c: detector_partial(iq, qx, qy, qz, x0, y0,
                                                       z0, c), chunks))
    return detector_epilogue(sum(parts), mirror), h, v


def detector_partial(iq, qx, qy, qz, x0, y0, z0, orients):
    """detector.py:278-300: the weighted sum over `orients` (a slice of
    orientation_list) of the gathered images, in list order.  Independent
    parts of the list may be summed on separate threads and added."""
    acc = np.zeros(x0.shape)
    for ps, pw, ph, hw, th, tw in orients:
        x, y, z = rotate_psi_phi_theta(x0, y0, z0, ps, ph, th)
        d = intersect_detector(iq, qx, qy, qz, x, y, z)
        d = d * (pw * hw * tw)
        acc += d
    return acc


def detector_epilogue(acc, mirror=True):
    """comparison.py:857-868: optional mirror, NaN/non-positive -> 1e-6,
    scale by 1e-6 (on a copy of the summed image)."""
    det = acc.copy()
    if mirror:
        det = mirror_vertical_horizontal(det)
    det[det != det] = 1e-6
    det[det <= 0] = 1e-6
    det *= 1e-6
    return det


# ------------------------------------------------------------------ slab
def slabmaker(cell_xyz, cell_elements, vecs, size):
    """comparison.py:595-671 (slabmaker_fitting) after the file is loaded:
    copies appended axis by axis (x, then y, then z) with the reference's
    float64 shift vectors, shift to the origin, crop to the central box,
    shift again.  vecs = (a, b, c) from calc_real_space_abc."""
    av, bv, cv = (np.asarray(v, dtype=np.float64) for v in vecs)
    coords = np.array(cell_xyz, dtype=np.float64)
    elements = np.asarray(cell_elements)
    x_size, y_size, z_size = size
    nx = int(np.ceil(2 * x_size / av[0]))
    ny = int(np.ceil(2 * y_size / bv[1]))
    nz = int(np.ceil(2 * z_size / cv[2]))
    for n, shift in ((nx, lambda i: np.array([av[0] * i, 0, 0])),
                     (ny, lambda i: np.array([bv[0] * i, bv[1] * i, 0])),
                     (nz, lambda i: np.array([cv[0] * i, cv[1] * i, cv[2] * i]))):
        base, base_el = coords.copy(), elements.copy()
        blocks, els = [coords], [elements]
        for i in range(n):
            blocks.append(base + shift(i + 1))
            els.append(base_el)
        coords = np.concatenate(blocks, axis=0)
        elements = np.concatenate(els, axis=0)
    ext = [np.max(coords[:, k]) - np.min(coords[:, k]) for k in range(3)]
    assert ext[0] > x_size, "x_max must be greater than x_size"
    assert ext[1] > y_size, "y_max must be greater than y_size"
    assert ext[2] > z_size, "z_max must be greater than z_size"
    buf = [(ext[0] - x_size) / 2, (ext[1] - y_size) / 2, (ext[2] - z_size) / 2]
    for k in range(3):
        coords[:, k] -= np.min(coords[:, k])
    keep = np.ones(len(coords), dtype=bool)
    for k in range(3):
        keep &= (coords[:, k] >= buf[k]) & (coords[:, k] <= ext[k] - buf[k])
    coords, elements = coords[keep], elements[keep]
    for k in range(3):
        coords[:, k] -= np.min(coords[:, k])
    return coords, elements


# ------------------------------------------------------------------ fit model
def fullfit_residuals(cell_xyz, cell_elements, vecs, size, r_voxel_size,
                      q_voxel_size, max_q, f_of_element, num_pixels,
                      angle_init_vals, angle_init_axs, psis, psi_w, phis, phi_w,
                      thetas, theta_w, rebin_map, rebin_mask, exp_qxy, exp_qz,
                      pad_width, pad_range, fill_bkg=False, smooth=0):
    """fit_slabsize.py:19-46 fullfit_model: slab, I(q) with the carbon f0,
    detector image (mirror=True), trim_sim_data (comparison.py:161-191),
    shift_peak, optimize_scale_offset (comparison.py:873-882, lstsq) and the
    residuals where the mask is 0, flattened."""
    coords, els = slabmaker(cell_xyz, cell_elements, vecs, size)
    fv = np.array([f_of_element[e] for e in els], dtype=complex)
    vg = voxelgrid([(coords, fv)], r_voxel_size, q_voxel_size, max_q, None,
                   fill_bkg, smooth)
    det, h, v = detector(vg["iq"], vg["qx"], vg["qy"], vg["qz"], num_pixels,
                         max_q, angle_init_vals, angle_init_axs, psis, psi_w,
                         phis, phi_w, thetas, theta_w, mirror=True)
    hm = (h >= np.min(exp_qxy)) & (h <= np.max(exp_qxy))
    vm = (v >= np.min(exp_qz)) & (v <= np.max(exp_qz))
    sim = det[vm, :][:, hm]
    sim = shift_peak(sim.copy(), h[hm], v[vm], pad_width, pad_range)
    keep = rebin_mask == 0
    A = np.vstack([sim[keep].ravel(), np.ones(int(keep.sum()))]).T
    (scale, offset), _, _, _ = np.linalg.lstsq(A, rebin_map[keep].ravel(), rcond=None)
    res = (rebin_map - (scale * sim + offset)) * keep
    return res.ravel(), scale, offset
