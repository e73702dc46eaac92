"""Differentiable detector image: torch.autograd.Function over the GB300
forward path and its hand-written adjoint kernels.

The reference (tools/comparison.py) fits simulated images to an experiment
by a scale + flat background least-squares misfit (optimize_scale_offset,
comparison.py:873-882) and explores parameters by brute force
(fit_slabsize.py).  This module gives the gradient of such a misfit with
respect to

  * per-atom occupancy (a real weight on each atom's scattering factor
    f = Z + f' + i f''; the structure's average voxel factor avg_voxel_f,
    which sets the smoothing background, follows the weighted factors as
    in comparison.py:744),
  * the smoothing sigma (in r-voxels, voxelgrids.py:364-379; continuous),
  * atom coordinates, with deposit="bilinear" (each atom split over the
    2 x 2 nearest cells; the nearest-bin deposit of the reference is
    piecewise constant in the coordinates).

Forward: voxel plan (deposit -> chirp-z transforms -> |F|^2 binning ->
I(q)) and detector plan on the GPU.  Backward: gw_detector_backward
(transposed epilogue, scatter over orientations) then gw_voxel_backward
(gather of dL/dsum, inverse transforms, gathers at the atoms), with the
slices recomputed from the atoms in batches of `checkpoint_every` phis.
The host adds the terms of the structure constants: avg_voxel_f depends on
the occupancies and on the slab volume (x_bound*y_bound*z_bound, through
the extreme atoms).  max_voxels, the smoothing plateau bounds and the
kernel radius are piecewise constant and contribute nothing.

PyTorch is used only for the autograd wrapper; all device work goes
through libgiwaxs_gb300.so.
"""
import numpy as np
import torch

from . import _native as N
from .forward import (DetectorPlan, VoxelGeometry, VoxelPlan, element_f_values,
                      structure_constants)


class DetectorModel:
    """coords (N,3), occupancy (N,), sigma -> detector image (n_v, n_h) of
    one structure, as voxelgridmaker_fitting + detectormaker_fitting compute
    it (comparison.py:673-870), with forward() and backward()."""

    def __init__(self, elements, energy, r_voxel_size, q_voxel_size, max_q,
                 num_pixels, angle_init_vals=(0, 0, 0),
                 angle_init_axs=("None", "None", "None"), psis=(0.0,),
                 psi_weights=None, det_phis=(0.0,), det_phi_weights=None,
                 thetas=(0.0,), theta_weights=None, mirror=True, phis=None,
                 deposit="nearest", checkpoint_every=16, f0_element="C",
                 f1f2=None, ctx=None):
        if deposit not in ("nearest", "bilinear"):
            raise ValueError("deposit must be 'nearest' or 'bilinear'")
        self.geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
        self.f_el = np.asarray(element_f_values(elements, energy, f1f2), complex)
        self.phis = (self.geom.auto_phis if phis is None
                     else np.asarray(phis, dtype=np.float64))
        self.deposit = deposit
        self.checkpoint_every = int(checkpoint_every)
        self.f0_element = f0_element
        # every plan of the model (the detector plan made here, the voxel
        # plans of each forward) works on one context, so that the I(q) a
        # voxel plan leaves on the device is ordered before the detector
        # reads it, whichever thread calls forward
        self.ctx = ctx or N.default_context()

        def w(a, ws):
            a = np.atleast_1d(np.asarray(a, dtype=np.float64))
            return a, (np.ones_like(a) / len(a) if ws is None
                       else np.asarray(ws, dtype=np.float64))

        psis, pw = w(psis, psi_weights)
        dphis, hw = w(det_phis, det_phi_weights)
        thetas, tw = w(thetas, theta_weights)
        q = self.geom.q_crop
        Qc = len(q)
        self.det = DetectorPlan((Qc, Qc, Qc), q, q, q, num_pixels, max_q,
                                angle_init_vals, angle_init_axs, psis, pw,
                                dphis, hw, thetas, tw, mirror=mirror, ctx=self.ctx)
        self._det_state = None

    @property
    def n_atoms(self):
        return len(self.f_el)

    def forward(self, coords, occupancy, sigma):
        """Detector image (float64) and the state backward() needs."""
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        occ = np.asarray(occupancy, dtype=np.float64)
        if coords.shape != (self.n_atoms, 3) or occ.shape != (self.n_atoms,):
            raise ValueError("coords must be (N,3) and occupancy (N,)")
        sigma = float(sigma)
        if sigma < 0:
            raise ValueError("sigma must be >= 0")
        f = self.f_el * occ
        plan = VoxelPlan(self.geom, [(coords, f, None)], phis=self.phis,
                         smooth=sigma, f0_element=self.f0_element,
                         batch_slices=self.checkpoint_every,
                         deposit=self.deposit, real=False, ctx=self.ctx)
        plan.set_atoms()
        plan.execute()
        self.det.set_iq_device32(plan.device_iq32())
        self.det.execute()
        img = self.det.result()
        state = dict(plan=plan, coords=coords, occ=occ, f=f, sigma=sigma)
        self._det_state = id(state)
        return img, state

    def backward(self, state, g_image, need_coords=True):
        """(dL/d occupancy (N,), dL/d sigma, dL/d coords (N,3) or None) from
        dL/d image."""
        plan = state["plan"]
        if self._det_state != id(state):
            # the detector plan last ran on another I(q): its epilogue mask
            # must be that of this state's image
            self.det.set_iq_device32(plan.device_iq32())
            self.det.execute()
            self._det_state = id(state)
        g_iq = plan.grad_buffer()
        self.det.backward(g_image, g_iq_device=g_iq)
        want_xyz = need_coords and self.deposit == "bilinear"
        out = plan.backward(g_iq, iq_on_device=True, want_xyz=want_xyz)
        coords, occ, f = state["coords"], state["occ"], state["f"]
        r = self.geom.r_voxel_size
        xb, yb, zb, avg, mv = structure_constants(coords, f, r)
        V = xb * yb * zb
        g_c = complex(out["g_c"][0])
        # avg_voxel_f = sum(f) r^3 / V, background constant c = avg * max_voxels
        g_fdep = out["g_f"] + g_c * (mv * r ** 3 / V)
        g_occ = (g_fdep.conj() * self.f_el).real
        g_xyz = None
        if want_xyz:
            g_xyz = out["g_xyz"].copy()
            # dL/dV through avg = sum(f) r^3 / V
            dLdV = (np.conj(g_c) * (mv * (-avg / V))).real
            for ax, other in ((0, yb * zb), (1, xb * zb), (2, xb * yb)):
                col = coords[:, ax]
                g_xyz[int(np.argmax(col)), ax] += dLdV * other
                g_xyz[int(np.argmin(col)), ax] -= dLdV * other
        return g_occ, out["g_sigma"], g_xyz

    def close(self):
        self.det.close()


class _DetectorImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, occupancy, sigma, coords, model):
        img, state = model.forward(coords.detach().cpu().numpy(),
                                   occupancy.detach().cpu().numpy(),
                                   float(sigma.detach().cpu()))
        ctx.model = model
        ctx.state = state
        ctx.dev = occupancy.device
        return torch.from_numpy(img).to(occupancy.device)

    @staticmethod
    def backward(ctx, g_img):
        need_occ, need_sigma, need_xyz = ctx.needs_input_grad[:3]
        g_occ, g_sigma, g_xyz = ctx.model.backward(
            ctx.state, g_img.detach().cpu().numpy(), need_coords=need_xyz)
        dev = ctx.dev
        return (torch.from_numpy(g_occ).to(dev) if need_occ else None,
                torch.tensor(g_sigma, dtype=torch.float64, device=dev)
                if need_sigma else None,
                torch.from_numpy(g_xyz).to(dev)
                if (need_xyz and g_xyz is not None) else None,
                None)


def detector_image(model, occupancy, sigma, coords):
    """Differentiable detector image (float64 tensor (n_v, n_h))."""
    if not torch.is_tensor(sigma):
        sigma = torch.tensor(float(sigma), dtype=torch.float64)
    return _DetectorImage.apply(occupancy, sigma, coords, model)


def scale_offset_misfit(sim, target, mask=None):
    """sum over unmasked pixels of (s*sim + b - target)^2 with (s, b) the
    least-squares scale and offset (comparison.py:873-882,
    optimize_scale_offset; mask == 1 marks excluded pixels as there).
    Returns (misfit, s, b)."""
    if mask is not None:
        keep = torch.as_tensor(np.asarray(mask) == 0, device=sim.device)
        x, t = sim[keep], target[keep]
    else:
        x, t = sim.reshape(-1), target.reshape(-1)
    n = x.numel()
    sx, st = x.sum(), t.sum()
    sxx, sxt = (x * x).sum(), (x * t).sum()
    det = n * sxx - sx * sx
    s = (n * sxt - sx * st) / det
    b = (st - s * sx) / n
    r = s * x + b - t
    return (r * r).sum(), s, b
