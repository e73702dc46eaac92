"""Drop-in stage drivers with the reference's signatures
(tools/comparison.py of the reference):

  voxelgridmaker_fitting   comparison.py:673-788  -> GPU voxel plan
  detectormaker_fitting    comparison.py:790-870  -> GPU detector plan
  slabmaker_fitting        comparison.py:595-671  (host: unit-cell tiling)
  optimize_scale_offset    comparison.py:873-882  (host least squares)

Keyword-only extensions (all default to the reference's behaviour):
  phis=            explicit rotation list instead of the automatic count
  mode=            'batched' (default) or 'plain' (per-rotation, full grid)
  accum=           'fp64' (default) or 'kahan32' accumulation
  exact=           detector: replay the float64 index chain for every sample
                   instead of only the samples the float32 path cannot decide
  weights=         per-atom occupancy multiplying the scattering factor
  ctx=             a giwaxsim_gb300._native.Context
"""
import numpy as np

from ..forward import (DetectorPlan, VoxelGeometry, VoxelPlan,
                       element_f_values)
from .utilities import calc_real_space_abc, load_pdb, load_xyz


def voxelgridmaker_fitting(coords, elements, r_voxel_size, q_voxel_size, max_q,
                           energy, num_cpus=None, fill_bkg=False, smooth=0, *,
                           phis=None, mode="batched", accum="fp64",
                           weights=None, f1f2=None, batch_slices=0, ctx=None):
    """I(q) on the cropped cube |q_i| < max_q + dq, C order (qy, qx, qz),
    with the carbon f0(q)^2 factor; returns (iq, qx, qy, qz) like the
    reference.  num_cpus is accepted and ignored (one GPU)."""
    geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
    coords = np.asarray(coords, dtype=np.float64)
    geom.check_bounds(coords)
    fv = element_f_values(elements, energy, f1f2)
    plan = VoxelPlan(geom, [(coords, fv, weights)], phis=phis,
                     fill_bkg=fill_bkg, smooth=smooth, mode=mode, accum=accum,
                     batch_slices=batch_slices, ctx=ctx)
    try:
        plan.set_atoms()
        plan.execute()
        iq = plan.iq()
    finally:
        plan.close()
    q = geom.q_crop
    return iq, q.copy(), q.copy(), q.copy()


def voxelgridmaker_average(structures, r_voxel_size, q_voxel_size, max_q,
                           energy, fill_bkg=False, smooth=0, *, phis=None,
                           accum="fp64", f1f2=None, batch_slices=0,
                           f0_element="C", ctx=None):
    """I(q) averaged over several structures before the f0 factor, as the
    legacy input_folder mode does (old_modules/voxelgridmaker.py:56-72).
    structures: list of (coords, elements) or (coords, elements, weights).
    All slices of all structures run in one batched plan."""
    geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
    items = []
    for s in structures:
        coords, elements = np.asarray(s[0], dtype=np.float64), s[1]
        w = s[2] if len(s) > 2 else None
        items.append((coords, element_f_values(elements, energy, f1f2), w))
    plan = VoxelPlan(geom, items, phis=phis, fill_bkg=fill_bkg, smooth=smooth,
                     accum=accum, average=True, f0_element=f0_element,
                     batch_slices=batch_slices, ctx=ctx)
    try:
        plan.set_atoms()
        plan.execute()
        iq = plan.iq()
    finally:
        plan.close()
    q = geom.q_crop
    return iq, q.copy(), q.copy(), q.copy()


def _weights(path, angles):
    return np.load(path) if path else np.ones_like(angles) / len(angles)


def detectormaker_fitting(iq, qx, qy, qz, num_pixels, max_q, angle_init_vals,
                          angle_init_axs, psis, psi_weights_path, phis,
                          phi_weights_path, thetas, theta_weights_path,
                          mirror=True, *, accum="fp64", exact=False,
                          ctx=None):
    """Detector image summed over psi x phi x theta orientations; returns
    (det_sum (num_pixels, num_pixels), det_h, det_v) like the reference."""
    psis, phis, thetas = (np.atleast_1d(np.asarray(a)) for a in (psis, phis, thetas))
    psi_w = _weights(psi_weights_path, psis)
    phi_w = _weights(phi_weights_path, phis)
    theta_w = _weights(theta_weights_path, thetas)
    assert len(psis) == len(psi_w), "psi weights length must equal psi_num"
    assert len(phis) == len(phi_w), "phi weights length must equal phi_num"
    assert len(thetas) == len(theta_w), "theta weights length must equal theta_num"
    assert np.abs(1 - np.sum(psi_w)) < 0.01, "psi weights must sum to 1"
    assert np.abs(1 - np.sum(phi_w)) < 0.01, "phi weights must sum to 1"
    assert np.abs(1 - np.sum(theta_w)) < 0.01, "theta weights must sum to 1"
    iq = np.asarray(iq)
    plan = DetectorPlan(iq.shape, qx, qy, qz, num_pixels, max_q,
                        angle_init_vals, angle_init_axs, psis, psi_w, phis,
                        phi_w, thetas, theta_w, mirror=mirror, accum=accum,
                        exact=exact, ctx=ctx)
    try:
        plan.set_iq(iq)
        plan.execute()
        det = plan.result()
    finally:
        plan.close()
    return det, plan.det_h.copy(), plan.det_v.copy()


def slabmaker_fitting(input_filepath, x_size, y_size, z_size, a, b, c, alpha,
                      beta, gamma):
    """Tile a unit cell into a slab of x/y/z size (comparison.py:595-671)."""
    if input_filepath.lower().endswith(".xyz"):
        coords, elements = load_xyz(input_filepath)
    elif input_filepath.lower().endswith(".pdb"):
        coords, elements = load_pdb(input_filepath)
    else:
        raise Exception("Files must be a .pdb or .xyz file")
    av, bv, cv = calc_real_space_abc(a, b, c, alpha, beta, gamma)
    nx = int(np.ceil(2 * x_size / av[0]))
    ny = int(np.ceil(2 * y_size / bv[1]))
    nz = int(np.ceil(2 * z_size / cv[2]))
    # the reference appends shifted copies axis by axis; keep its order
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


def optimize_scale_offset(sim_map, rebin_map, rebin_mask):
    """Least-squares scale and offset of sim onto rebin where mask == 0."""
    sim = sim_map[rebin_mask == 0].ravel()
    reb = rebin_map[rebin_mask == 0].ravel()
    A = np.vstack([sim, np.ones_like(sim)]).T
    coeffs, _, _, _ = np.linalg.lstsq(A, reb, rcond=None)
    return coeffs[0], coeffs[1]
