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

Not provided: shift_peak (the reference's polar-warp padding of the pi-pi
peak, comparison.py:566-592); the simulated image is compared as trimmed.
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
                 mirror=True, f1f2=None, ctx=None):
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
        self.cmp = Comparison(self.det.det_h, self.det.det_v, exp_img, exp_qxy,
                              exp_qz, exp_mask, ctx=self.ctx)
        self.evaluations = 0

    def images(self, sizes):
        """Detector images (host) of slabs of the given (x, y, z) sizes."""
        return [img for img, _ in self._run(sizes, keep_images=True)]

    def misfits(self, sizes):
        """(scale, offset, misfit) of each candidate (x, y, z) size; all
        candidates in one batched voxel pass."""
        return [m for _, m in self._run(sizes, keep_images=False)]

    def _run(self, sizes, keep_images):
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
                s, o, mis, _ = self.cmp.evaluate(self.det.device_result(),
                                                 on_device=True)
                img = self.det.result() if keep_images else None
                out.append((img, (s, o, mis)))
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
