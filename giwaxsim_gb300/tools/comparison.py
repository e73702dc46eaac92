"""Drop-in stage drivers with the reference's signatures
(tools/comparison.py of the reference):

  voxelgridmaker_fitting   comparison.py:673-788  -> GPU voxel plan
  detectormaker_fitting    comparison.py:790-870  -> GPU detector plan
  slabmaker_fitting        comparison.py:595-671  -> GPU slab (gw_slab)
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

from ..forward import (DetectorPlan, Slab, VoxelGeometry, VoxelPlan,
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
                      beta, gamma, *, ctx=None):
    """Tile a unit cell into a slab of x/y/z size (comparison.py:595-671),
    on the device (gw_slab): same coordinates bit for bit, same atom order,
    same AssertionError messages."""
    if input_filepath.lower().endswith(".xyz"):
        coords, elements = load_xyz(input_filepath)
    elif input_filepath.lower().endswith(".pdb"):
        coords, elements = load_pdb(input_filepath)
    else:
        raise Exception("Files must be a .pdb or .xyz file")
    vecs = np.array(calc_real_space_abc(a, b, c, alpha, beta, gamma))
    slab = Slab(coords, vecs, (x_size, y_size, z_size), ctx=ctx)
    try:
        xyz, src = slab.coords()
    finally:
        slab.close()
    return xyz, np.asarray(elements)[src]


def optimize_scale_offset(sim_map, rebin_map, rebin_mask):
    """Least-squares scale and offset of sim onto rebin where mask == 0."""
    sim = sim_map[rebin_mask == 0].ravel()
    reb = rebin_map[rebin_mask == 0].ravel()
    A = np.vstack([sim, np.ones_like(sim)]).T
    coeffs, _, _, _ = np.linalg.lstsq(A, reb, rcond=None)
    return coeffs[0], coeffs[1]
