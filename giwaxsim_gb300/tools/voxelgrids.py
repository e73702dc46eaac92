"""Drop-in for the reference's tools/voxelgrids.py, on the GB300 library.

  downselect_voxelgrid         voxelgrids.py:16-48   (index arithmetic only)
  rectangular_collapse_lengths voxelgrids.py:238-309 -> gw_collapse_lengths
  rotate_project_fft_coords    voxelgrids.py:311-416 -> one-slice plain plan,
                               accumulated into the named shared-memory grids
  process_file2                voxelgrids.py:464-506 -> gw_bin_slice
  generate_voxel_grid_low_mem  voxelgrids.py:535-722 (aff_num_qs >= 1; the
                               multi-q shells -> gw_voxel_set_shells)
  add_f0_q_3d                  voxelgrids.py:828-857 -> gw_f0_scale

The per-slice functions keep the reference's calling convention (shared
memory by name) for callers that drive slices one at a time; the batched
voxelgridmaker_fitting in tools/comparison.py is the fast path.  The
reference calls them from a thread pool and its unguarded accumulation into
the shared grids loses updates; here the device work of concurrent calls
overlaps (one context per thread) and the additions into the named grids
are serialised within the process, so a threaded run sums what a serial
run sums.
"""
import ctypes
import os
import threading
from multiprocessing import shared_memory

import numpy as np

from .. import _native as N
from ..forward import VoxelGeometry, VoxelPlan, element_f_values
from .ptable_dict import aff_dict, ptable
from .utilities import (get_element_f0_dict, get_element_f1_f2_dict, load_pdb,
                        load_xyz)


def _axes_identical(qx, qy, qz):
    if not (np.array_equal(qx, qy) and np.array_equal(qx, qz)):
        raise ValueError("qx, qy and qz must be the same axis (the reference "
                         "builds them as one linspace)")


def downselect_voxelgrid(grid, x_axis, y_axis, z_axis, max_val):
    """Cube of `grid` (y, x, z) with |q| < max_val + voxel size per axis."""
    voxel = np.abs(x_axis[1] - x_axis[0])
    max_val = max_val + voxel
    xi = np.where(np.abs(x_axis) < max_val)[0]
    yi = np.where(np.abs(y_axis) < max_val)[0]
    zi = np.where(np.abs(z_axis) < max_val)[0]
    return (grid[yi[0]:yi[-1] + 1, xi[0]:xi[-1] + 1, zi[0]:zi[-1] + 1],
            x_axis[xi[0]:xi[-1] + 1], y_axis[yi[0]:yi[-1] + 1],
            z_axis[zi[0]:zi[-1] + 1])


def _phi_struct(phi):
    g = VoxelGeometry.__new__(VoxelGeometry)
    g.h_max = 0.0
    return VoxelGeometry.phi_table(g, np.array([phi], dtype=np.float64))


def rectangular_collapse_lengths(x_vals, hor_length, ver_length, phi,
                                 ctx=None):
    """Path length through the slab's x-y rectangle rotated by phi, per
    column position."""
    ctx = ctx or N.default_context()
    x = np.ascontiguousarray(x_vals, dtype=np.float64)
    out = np.empty_like(x)
    t = _phi_struct(phi)
    N.check(N.lib().gw_collapse_lengths(ctx.handle, N.ptr(x), len(x),
                                        float(hor_length), float(ver_length),
                                        N.ptr(t), N.ptr(out)))
    return out


# held while a slice's sums and counts are added into the named grids
_GRID_ADD_LOCK = threading.Lock()


def _shm_grid(name, q_num):
    shm = shared_memory.SharedMemory(name=name)
    return shm, np.ndarray((q_num,) * 3, dtype=np.float64, buffer=shm.buf)


def rotate_project_fft_coords(args, ctx=None):
    """One phi slice -> its |F|^2 binned into the named (sum, count) grids
    (voxelgrids.py:311-416).  args is the reference's 16-tuple."""
    (coords, f_values, phi, grid_size, r_voxel_size, avg_voxel_f, x_bound,
     y_bound, z_bound, fill_bkg, smooth, qx, qy, qz, sum_name,
     count_name) = args
    _axes_identical(qx, qy, qz)
    geom = VoxelGeometry.from_axes(grid_size, r_voxel_size, qx)
    plan = VoxelPlan(geom, [(coords, f_values, None)], phis=[phi],
                     fill_bkg=fill_bkg, smooth=smooth, mode="plain",
                     f0_element=None,
                     constants=[(x_bound, y_bound, z_bound, avg_voxel_f)],
                     ctx=ctx)
    try:
        plan.set_atoms()
        plan.execute()
        sums, counts = plan.sums(), plan.counts()
    finally:
        plan.close()
    q_num = len(qx)
    s_shm, s = _shm_grid(sum_name, q_num)
    c_shm, c = _shm_grid(count_name, q_num)
    try:
        with _GRID_ADD_LOCK:
            s += sums
            c += counts
    finally:
        del s, c
        s_shm.close()
        c_shm.close()


def process_file2(iq_2d, det_h_qx, det_h_qy, det_v_qz, qx, qy, qz,
                  voxel_grid_shm_name, voxel_grid_count_shm_name, ctx=None):
    """Bin one |F|^2 slice into the named (sum, count) grids
    (voxelgrids.py:464-506)."""
    ctx = ctx or N.default_context()
    _axes_identical(qx, qy, qz)
    iq_2d = np.ascontiguousarray(iq_2d, dtype=np.float64)
    hx = np.ascontiguousarray(det_h_qx, dtype=np.float64)
    hy = np.ascontiguousarray(det_h_qy, dtype=np.float64)
    vz = np.ascontiguousarray(det_v_qz, dtype=np.float64)
    q_num = len(qx)
    s_shm, s = _shm_grid(voxel_grid_shm_name, q_num)
    c_shm, c = _shm_grid(voxel_grid_count_shm_name, q_num)
    try:
        # gw_bin_slice adds into the grids on the host after its device pass
        with _GRID_ADD_LOCK:
            N.check(N.lib().gw_bin_slice(
                ctx.handle, N.ptr(iq_2d), iq_2d.shape[0], iq_2d.shape[1],
                N.ptr(hx), N.ptr(hy), N.ptr(vz), q_num, float(np.min(qx)),
                float(np.max(qx)), float(np.diff(qz)[0]), N.ptr(s), N.ptr(c)))
    finally:
        del s, c
        s_shm.close()
        c_shm.close()


def add_f0_q_3d(iq, qx_axis, qy_axis, qz_axis, element, ctx=None):
    """iq times the normalised f0(|q|)^2 of `element` (voxelgrids.py:828-857)."""
    ctx = ctx or N.default_context()
    iq = np.ascontiguousarray(iq, dtype=np.float64)
    out = np.empty_like(iq)
    shape = np.array(iq.shape, dtype=np.int32)
    coef = np.ascontiguousarray(aff_dict[element], dtype=np.float64)
    qx, qy, qz = (np.ascontiguousarray(a, dtype=np.float64)
                  for a in (qx_axis, qy_axis, qz_axis))
    N.check(N.lib().gw_f0_scale(ctx.handle, N.ptr(iq), N.ptr(shape), N.ptr(qx),
                                N.ptr(qy), N.ptr(qz), N.ptr(coef),
                                float(ptable[element]), N.ptr(out)))
    return out


def aff_shell_tables(q_axis, aff_num_qs, elements, energy, f1f2=None):
    """Shell bounds and per-shell atom f values of the multi-q branch
    (voxelgrids.py:659-669): K = aff_num_qs shells of width
    step = max_q_diag / K over (0, max_q_diag], shell k centred at
    q_k = step/2 + k step, atoms scattering with f0(q_k) + f' + i f''.
    Returns (lower, upper, f (K, n_atoms) complex)."""
    K = int(aff_num_qs)
    max_q_diag = q_axis[-1]
    step = max_q_diag / K
    elements = np.asarray(elements)
    d = f1f2 if f1f2 is not None else get_element_f1_f2_dict(energy, elements)
    lower, upper, f = [], [], []
    for k in range(K):
        q_val = 0.5 * step + k * step
        upper.append(q_val + step / 2)
        lower.append(q_val - step / 2)
        f0 = get_element_f0_dict(q_val, elements)
        f.append(np.array([f0[e] for e in elements])
                 + np.array([d[e] for e in elements]))
    return np.array(lower), np.array(upper), np.array(f, dtype=complex)


def generate_voxel_grid_low_mem(input_path, r_voxel_size, q_voxel_size, max_q,
                                aff_num_qs, energy, gen_name, output_dir=None,
                                scratch_folder=None, num_cpus=None,
                                fill_bkg=False, smooth=0, *, phis=None,
                                aff_mode="reference", f1f2=None, ctx=None):
    """Full q_num^3 I(q) of one structure file (voxelgrids.py:535-722).

    aff_num_qs > 1 evaluates the atomic form factors per q shell
    (voxelgrids.py:650-707).  aff_mode "reference" returns what the
    reference returns: its loop overwrites the grid with every shell's I(q)
    and adds the shell-masked grid to itself (:703-707), i.e. the last
    shell's I(q) over the whole grid, doubled inside the last shell.
    aff_mode "per_shell" gives each voxel the I(q) of its own shell (the
    evident intent; 0 outside every shell), in one device pass per shell.
    f1f2: element -> f' + i f'' (default: the xraydb lookup)."""
    if int(aff_num_qs) < 1:
        raise Exception("Invalid aff_num_qs value. Must be non-negative integer")
    if aff_mode not in ("reference", "per_shell"):
        raise ValueError("aff_mode must be 'reference' or 'per_shell'")
    geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
    if input_path[-3:] == "xyz":
        coords, elements = load_xyz(input_path)
    elif input_path[-3:] == "pdb":
        coords, elements = load_pdb(input_path)
    else:
        raise Exception("files must be a .pdb or .xyz file")
    geom.check_bounds(coords)
    full = VoxelGeometry.from_axes(geom.grid_size, r_voxel_size, geom.q)
    fv = element_f_values(elements, energy, f1f2)
    plan = VoxelPlan(full, [(coords, fv, None)],
                     phis=geom.auto_phis if phis is None else phis,
                     fill_bkg=fill_bkg, smooth=smooth, f0_element=None,
                     real=False if int(aff_num_qs) > 1 else None, ctx=ctx)
    try:
        plan.set_atoms()
        if int(aff_num_qs) > 1:
            lower, upper, fk = aff_shell_tables(geom.q, aff_num_qs, elements,
                                                energy, f1f2)
            r3 = r_voxel_size ** 3
            b = plan.structs[0]
            vol = b["x_bound"] * b["y_bound"] * b["z_bound"]
            avg = np.array([[(np.sum(f) / vol) * r3] for f in fk])
            plan.set_shells(geom.q, lower, upper, fk, avg, mode=aff_mode)
        plan.execute()
        iq = plan.iq()
    finally:
        plan.close()
    q = geom.q
    if output_dir:
        save_path = f"{output_dir}/{gen_name}_output_files/"
        os.makedirs(save_path, exist_ok=True)
        np.save(f"{save_path}{gen_name}_iq.npy", iq)
        for ax in ("qx", "qy", "qz"):
            np.save(f"{save_path}{gen_name}_{ax}.npy", q)
        return None
    return iq, q, q, q
