"""Slab-size fitting on the GPU path (fit_slabsize.py of the reference).

The reference fits the slab's x/y/z size to an experimental image with
lmfit's Nelder-Mead, and every evaluation rebuilds slab, I(q) and detector
image on the CPU (fit_slabsize.py:18-46, :133-173).  Here one evaluation of
K candidate sizes is one pass: K slabs tiled on the device (gw_slab), one
batched voxel plan with a separate I(q) per candidate (GW_STRUCTS_SEPARATE:
all K x n_phi slices in one graph), a detector image per candidate from a
detector plan made once, and the scale + offset comparison against the
experiment, rebinned once (gw_compare).  Optimisers:

  method="nelder-mead"  scipy's Nelder-Mead on the varied sizes (the
                        reference's lmfit method), one candidate per pass;
  method="grid"         rounds of K candidates evaluated together on a
                        shrinking grid around the best one.

shift=(pad_width, pad_range) applies shift_peak (the polar-warp padding of
the pi-pi peak, comparison.py:566-592) to every trimmed image on the device
before the comparison, as fullfit_model does (fit_slabsize.py:36).

fullfit_model below keeps the reference's signature and return value (the
residual vector lmfit minimises) and runs on a cached SlabFit.
"""
import itertools

import numpy as np

from . import _native as N
from .forward import DetectorPlan, Slab, VoxelGeometry, VoxelPlan, element_f_values
from .tools.comparison import Comparison
from .tools.utilities import calc_real_space_abc


class SlabFit:
    def __init__(self, cell_xyz, cell_elements, cell_params, r_voxel_size,
                 q_voxel_size, max_q, energy, num_pixels, exp_img, exp_qxy,
                 exp_qz, exp_mask, fill_bkg=False, smooth=0, phis=None,
                 angle_init_vals=(0, 0, 0), angle_init_axs=("None",) * 3,
                 psis=(0.0,), psi_weights=None, det_phis=(0.0,),
                 det_phi_weights=None, thetas=(0.0,), theta_weights=None,
                 mirror=True, f1f2=None, shift=None, rebinned=False, ctx=None):
        """rebinned=True: exp_img / exp_mask are already on the trimmed
        simulation grid (rebin_map / rebin_mask of fit_slabsize.py:140-142)."""
        self.ctx = ctx or N.default_context()
        self.cell_xyz = np.asarray(cell_xyz, dtype=np.float64)
        self.cell_f = element_f_values(cell_elements, energy, f1f2)
        self.vecs = np.array(calc_real_space_abc(*cell_params))
        self.geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
        self.phis = phis
        self.fill_bkg, self.smooth = fill_bkg, smooth

        def w(a, ws):
            a = np.atleast_1d(np.asarray(a, dtype=np.float64))
            return a, (np.ones_like(a) / len(a) if ws is None else np.asarray(ws))

        psis, pw = w(psis, psi_weights)
        dph, hw = w(det_phis, det_phi_weights)
        th, tw = w(thetas, theta_weights)
        q = self.geom.q_crop
        Qc = len(q)
        self.det = DetectorPlan((Qc,) * 3, q, q, q, num_pixels, max_q,
                                angle_init_vals, angle_init_axs, psis, pw, dph,
                                hw, th, tw, mirror=mirror, ctx=self.ctx)
        weights = None
        if rebinned:
            from .tools.comparison import _identity
            weights = _identity(np.shape(exp_img))
        self.cmp = Comparison(self.det.det_h, self.det.det_v, exp_img, exp_qxy,
                              exp_qz, exp_mask, weights=weights, shift=shift,
                              ctx=self.ctx)
        self.evaluations = 0

    def images(self, sizes):
        """Detector images (host) of slabs of the given (x, y, z) sizes."""
        return [img for img, _ in self._run(sizes, keep_images=True)]

    def misfits(self, sizes):
        """(scale, offset, misfit) of each candidate (x, y, z) size; all
        candidates in one batched voxel pass."""
        return [m for _, m in self._run(sizes, keep_images=False)]

    def residuals(self, size):
        """The residual map of one candidate (fit_slabsize.py:43-44)."""
        return self._run([size], keep_images=False, residual=True)[0][1][3]

    def _run(self, sizes, keep_images, residual=False):
        sizes = [tuple(float(v) for v in s) for s in sizes]
        items = []
        for s in sizes:
            slab = Slab(self.cell_xyz, self.vecs, s, ctx=self.ctx)
            try:
                xyz, src = slab.coords()
            finally:
                slab.close()
            self.geom.check_bounds(xyz)
            items.append((xyz, self.cell_f[src], None))
        plan = VoxelPlan(self.geom, items, phis=self.phis,
                         fill_bkg=self.fill_bkg, smooth=self.smooth,
                         average="separate", ctx=self.ctx)
        out = []
        try:
            plan.set_atoms()
            plan.execute()
            for k in range(len(sizes)):
                self.det.set_iq_device32(plan.device_iq32(k))
                self.det.execute()
                r = self.cmp.evaluate(self.det.device_result(), on_device=True,
                                      residual=residual)
                img = self.det.result() if keep_images else None
                out.append((img, r[:3] + (r[4],) if residual else r[:3]))
        finally:
            plan.close()
        self.evaluations += len(sizes)
        return out

    def fit(self, init_size, vary=(True, True, True), bounds=None,
            max_evals=50, method="nelder-mead", grid_points=3, rounds=4,
            step=0.15):
        """Best (x, y, z) size and its misfit.  bounds: per-axis (lo, hi),
        default (25, 3 x initial) as fit_slabsize.py:152-154 sets them."""
        init = np.asarray(init_size, dtype=np.float64)
        vary = np.asarray(vary, dtype=bool)
        if bounds is None:
            bounds = [(25.0, 3.0 * v) for v in init]
        lo = np.array([b[0] for b in bounds])
        hi = np.array([b[1] for b in bounds])
        history = []

        def full(x):
            s = init.copy()
            s[vary] = np.clip(x, lo[vary], hi[vary])
            return s

        if method == "nelder-mead":
            from scipy.optimize import minimize

            class _Spent(Exception):
                pass

            def f(x):
                if len(history) >= max_evals:  # a hard cap on evaluations
                    raise _Spent
                s = full(x)
                m = self.misfits([s])[0][2]
                history.append((tuple(s), m))
                return m

            try:
                minimize(f, init[vary], method="Nelder-Mead",
                         bounds=list(zip(lo[vary], hi[vary])),
                         options={"maxfev": max_evals})
            except _Spent:
                pass
        elif method == "grid":
            center = init[vary].copy()
            width = step * center
            for _ in range(rounds):
                axes = [np.linspace(c - w_, c + w_, grid_points)
                        for c, w_ in zip(center, width)]
                cands = [full(np.array(p)) for p in itertools.product(*axes)]
                ms = self.misfits(cands)
                for s, m in zip(cands, ms):
                    history.append((tuple(s), m[2]))
                best = cands[int(np.argmin([m[2] for m in ms]))]
                center = best[vary]
                width = width / (grid_points - 1)
        else:
            raise ValueError("method must be 'nelder-mead' or 'grid'")
        best_size, best_m = min(history, key=lambda h: h[1])
        return dict(size=best_size, misfit=best_m, evaluations=len(history),
                    history=history)

    def close(self):
        self.det.close()
        self.cmp.close()


_MODELS = {}


def _model_key(*parts):
    import hashlib
    h = hashlib.sha256()
    for p in parts:
        a = np.asarray(p) if not isinstance(p, str) else None
        if a is not None and a.dtype != object:
            h.update(str(a.dtype).encode() + str(a.shape).encode())
            h.update(np.ascontiguousarray(a).tobytes())
        else:
            h.update(repr(p).encode())
    return h.hexdigest()


def fullfit_model(params, fixed_slab_params, fixed_voxelgrid_params,
                  fixed_detectormaker_params, fixed_exp_params, *, ctx=None):
    """fit_slabsize.py:19-46 with the reference's arguments and return value
    (the residual vector, flattened, that lmfit minimises): slab of
    params['x_size'/'y_size'/'z_size'], I(q), detector image (mirror=True),
    trim, shift_peak, scale + offset, residuals where rebin_mask == 0.  The
    device plans of one set of fixed parameters are made on the first call
    and reused."""
    from .tools.utilities import load_pdb, load_xyz
    size = tuple(float(params[k]) for k in ("x_size", "y_size", "z_size"))
    input_filepath, a, b, c, alpha, beta, gamma = fixed_slab_params
    r_voxel_size, q_voxel_size, max_q, energy, fill_bkg, smooth = fixed_voxelgrid_params
    (num_pixels, angle_init_vals, angle_init_axs, psis, psi_weights_path, phis,
     phi_weights_path, thetas, theta_weights_path) = fixed_detectormaker_params
    rebin_map, rebin_mask, exp_qxy, exp_qz, pad_width, pad_range = fixed_exp_params
    key = _model_key(input_filepath, (a, b, c, alpha, beta, gamma),
                     fixed_voxelgrid_params, num_pixels, angle_init_vals,
                     angle_init_axs, psis, psi_weights_path, phis,
                     phi_weights_path, thetas, theta_weights_path, rebin_map,
                     rebin_mask, exp_qxy, exp_qz, pad_width, pad_range, id(ctx))
    fit = _MODELS.get(key)
    if fit is None:
        if input_filepath.lower().endswith(".xyz"):
            cell_xyz, cell_el = load_xyz(input_filepath)
        elif input_filepath.lower().endswith(".pdb"):
            cell_xyz, cell_el = load_pdb(input_filepath)
        else:
            raise Exception("Files must be a .pdb or .xyz file")

        def wts(path, ang):
            ang = np.atleast_1d(np.asarray(ang, dtype=np.float64))
            return ang, (np.load(path) if path else np.ones_like(ang) / len(ang))

        ps, pw = wts(psi_weights_path, psis)
        ph, hw = wts(phi_weights_path, phis)
        th, tw = wts(theta_weights_path, thetas)
        if len(_MODELS) >= 4:
            for m in _MODELS.values():
                m.close()
            _MODELS.clear()
        fit = _MODELS[key] = SlabFit(
            cell_xyz, cell_el, (a, b, c, alpha, beta, gamma), r_voxel_size,
            q_voxel_size, max_q, energy, num_pixels, rebin_map, exp_qxy, exp_qz,
            rebin_mask, fill_bkg=fill_bkg, smooth=smooth,
            angle_init_vals=angle_init_vals, angle_init_axs=angle_init_axs,
            psis=ps, psi_weights=pw, det_phis=ph, det_phi_weights=hw,
            thetas=th, theta_weights=tw, mirror=True,
            shift=(pad_width, pad_range), rebinned=True, ctx=ctx)
    return fit.residuals(size).ravel()
