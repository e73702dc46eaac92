"""TEST INFRASTRUCTURE ONLY -- dense float64 PyTorch restatement of the
differentiable detector model, the reference gradient for the adjoint
kernels.

Every slice is the full g x g complex128 grid (no chirp-z, no window, no
band): atoms deposited with index_put (nearest bin, as
tools/voxelgrids.py:328-341, or bilinear), background and Gaussian
smoothing as voxelgrids.py:364-379 (sigma a tensor, continuous), fft2,
fftshift, |.|^2 (voxelgrids.py:382-392), binning into the cropped cube
(voxelgrids.py:464-506), divide/f0 (comparison.py:765-786), orientation sum
and epilogue (comparison.py:790-870).  Index arithmetic (floor divisions,
detector gathers, bin indices) comes from the numpy oracle, so it is the
reference's; values are torch float64 functions of (occupancy, sigma,
coords) and torch autograd differentiates them.

gradient() runs the adjoint in the same two phases the GPU path uses:
dL/dsum from the summed grid, then the slices again in chunks.
"""
import math

import numpy as np
import torch

from oracle import giwaxs_oracle as O


class DenseModel:
    def __init__(self, elements_f, r, dq, max_q, phis, num_pixels,
                 angle_init_vals, angle_init_axs, psis, psi_weights=None,
                 mirror=True, deposit="nearest", f0_element="C",
                 device="cpu"):
        self.f = torch.as_tensor(np.asarray(elements_f, complex),
                                 dtype=torch.complex128, device=device)
        self.r = float(r)
        self.deposit = deposit
        self.device = device
        self.phis = np.asarray(phis, dtype=np.float64)
        g, q, _ = O.voxel_geometry(r, dq, max_q)
        self.g, self.q = g, q
        voxel = abs(q[1] - q[0])
        keep = np.where(np.abs(q) < max_q + voxel)[0]
        self.lo, self.hi = int(keep[0]), int(keep[-1])
        self.Qc = self.hi - self.lo + 1
        qc = q[self.lo:self.hi + 1]
        self.qc = qc
        # binning tables per slice and the count grid
        Qc = self.Qc
        cnt = np.zeros(Qc ** 3)
        self.bins = []
        for phi in self.phis:
            hx, hy, vz = O.slice_axes(g, r, phi)
            vm, hm, iy, ix, iz = O.bin_indices(hx, hy, vz, q, q, q)
            rows = np.where(vm)[0]
            cols = np.where(hm)[0]
            rk = (iz >= self.lo) & (iz <= self.hi)
            ck = ((iy >= self.lo) & (iy <= self.hi) & (ix >= self.lo)
                  & (ix <= self.hi))
            rows, iz = rows[rk], iz[rk] - self.lo
            cols = cols[ck]
            base = ((iy[ck] - self.lo) * Qc + (ix[ck] - self.lo)) * Qc
            flat = (base[None, :] + iz[:, None]).ravel()
            np.add.at(cnt, flat, 1.0)
            self.bins.append((torch.as_tensor(rows, device=device),
                              torch.as_tensor(cols, device=device),
                              torch.as_tensor(flat, device=device)))
        f0 = O.f0_factor(qc, qc, qc, f0_element).ravel()
        scale = np.where(cnt > 0, f0 / np.where(cnt > 0, cnt, 1), 0.0)
        self.scale = torch.as_tensor(scale, device=device)
        # detector gathers
        x0, y0, z0, h, v = O.init_detector(num_pixels, max_q, angle_init_vals,
                                           angle_init_axs)
        psis = np.atleast_1d(np.asarray(psis, dtype=np.float64))
        pw = (np.ones_like(psis) / len(psis) if psi_weights is None
              else np.asarray(psi_weights))
        idx, w = [], []
        for ps, wt in zip(psis, pw):
            x, y, z = O.rotate_psi_phi_theta(x0, y0, z0, ps, 0.0, 0.0)
            iy, ix, iz = O.intersect_indices((Qc,) * 3, qc, qc, qc, x, y, z)
            idx.append((iy * Qc + ix) * Qc + iz)
            w.append(wt)
        self.det_idx = torch.as_tensor(np.stack(idx), device=device)
        self.det_w = torch.as_tensor(np.asarray(w, dtype=np.float64), device=device)
        self.npix = num_pixels
        self.mirror = mirror

    # ---------------------------------------------------------- forward
    def constants(self, coords, occ):
        """avg_voxel_f * max_voxels (comparison.py:712-744,
        voxelgrids.py:344) as a tensor function of coords and occ."""
        ext = coords.amax(0) - coords.amin(0)
        V = ext[0] * ext[1] * ext[2]
        fsum = (self.f * occ.to(torch.complex128)).sum()
        avg = fsum / V * self.r ** 3
        xb, yb = float(ext[0].detach()), float(ext[1].detach())
        mv = math.sqrt(xb ** 2 + yb ** 2) // self.r
        return avg * mv

    def slice_intensity(self, coords, occ, sigma, c, k):
        """|fftshift(fft2(grid))|^2 of slice k (torch, differentiable)."""
        g, r = self.g, self.r
        phi = self.phis[k]
        cn = coords.detach().cpu().numpy()
        rot = O.rotate_coords_z(cn, phi)
        ry = rot[:, 1] - np.min(rot[:, 1])
        rz = rot[:, 2] - np.min(rot[:, 2])
        yi = (ry // r).astype(np.int64)
        zi = (rz // r).astype(np.int64)
        ok = (yi >= 0) & (yi < g) & (zi >= 0) & (zi < g)
        pr = np.radians(phi)
        yt = coords[:, 0] * float(np.sin(pr)) + coords[:, 1] * float(np.cos(pr))
        zt = coords[:, 2]
        fv = self.f * occ.to(torch.complex128)
        grid = torch.zeros((g, g), dtype=torch.complex128, device=self.device)
        okt = torch.as_tensor(ok, device=self.device)
        yit = torch.as_tensor(yi, device=self.device)
        zit = torch.as_tensor(zi, device=self.device)
        if self.deposit == "nearest":
            grid.index_put_((zit[okt], yit[okt]), fv[okt], accumulate=True)
        else:
            fu = (yt - yt.min()) / r - yit
            fz = (zt - zt.min()) / r - zit
            for dz in (0, 1):
                wz = fz if dz else 1 - fz
                for dy in (0, 1):
                    wy = fu if dy else 1 - fu
                    zc, yc = zit + dz, yit + dy
                    m = okt & (zc < g) & (yc < g)
                    grid.index_put_((zc[m], yc[m]), (fv * (wz * wy))[m],
                                    accumulate=True)
        if float(sigma) > 0:
            ylo, yhi = int(yi[ok].min()), int(yi[ok].max())
            zlo, zhi = int(zi[ok].min()), int(zi[ok].max())
            my = self._profile(ylo, yhi, sigma)
            mz = self._profile(zlo, zhi, sigma)
            M = mz[:, None] * my[None, :]
            grid = (grid - c) * M + c
        F = torch.fft.fftshift(torch.fft.fft2(grid))
        return F.real ** 2 + F.imag ** 2

    def _profile(self, lo, hi, sigma):
        g = self.g
        s, e = O.mask_bounds(lo, hi, float(sigma), g)
        mask = torch.zeros(g, dtype=torch.float64, device=self.device)
        mask[s:e] = 1.0
        radius = int(4.0 * float(sigma) + 0.5)
        j = torch.arange(-radius, radius + 1, dtype=torch.float64, device=self.device)
        w = torch.exp(-0.5 * j * j / (sigma * sigma))
        w = w / w.sum()
        out = torch.zeros(g, dtype=torch.float64, device=self.device)
        for t in range(-radius, radius + 1):
            out = out + w[t + radius] * torch.roll(mask, shifts=-t)
        return out

    def bin_slice(self, I, k):
        rows, cols, flat = self.bins[k]
        return I[rows][:, cols].reshape(-1), flat

    def summed(self, coords, occ, sigma):
        c = self.constants(coords, occ)
        s = torch.zeros(self.Qc ** 3, dtype=torch.float64, device=self.device)
        for k in range(len(self.phis)):
            vals, flat = self.bin_slice(self.slice_intensity(coords, occ, sigma, c, k), k)
            s = s.index_add(0, flat, vals)
        return s

    def image_from_sum(self, s):
        iq = s * self.scale
        det = (iq[self.det_idx] * self.det_w[:, None]).sum(0)
        det = det.reshape(self.npix, self.npix)
        if self.mirror:
            det = det + det.flip(1) + det.flip(0) + det.flip(0).flip(1)
        det = torch.where(det > 0, det, torch.full_like(det, 1e-6))
        return det * 1e-6

    def image(self, coords, occ, sigma):
        with torch.no_grad():
            return self.image_from_sum(self.summed(coords, occ, sigma))

    # ---------------------------------------------------------- gradient
    def gradient(self, loss_fn, coords, occ, sigma, chunk=16):
        """(loss, dL/docc, dL/dsigma, dL/dcoords) for loss_fn(image)."""
        with torch.no_grad():
            s = self.summed(coords, occ, sigma)
        s = s.clone().requires_grad_(True)
        loss = loss_fn(self.image_from_sum(s))
        (gs,) = torch.autograd.grad(loss, s)
        occ = occ.detach().clone().requires_grad_(True)
        sigma = sigma.detach().clone().requires_grad_(True)
        coords = coords.detach().clone().requires_grad_(True)
        for k0 in range(0, len(self.phis), chunk):
            c = self.constants(coords, occ)
            acc = 0.0
            for k in range(k0, min(k0 + chunk, len(self.phis))):
                vals, flat = self.bin_slice(
                    self.slice_intensity(coords, occ, sigma, c, k), k)
                acc = acc + (vals * gs[flat]).sum()
            acc.backward()
        def g(t):  # a parameter the loss does not depend on has no grad
            return torch.zeros_like(t) if t.grad is None else t.grad.detach()

        return float(loss), g(occ), g(sigma), g(coords)


def misfit(sim, target):
    """sum (s*sim + b - target)^2 with the least-squares (s, b)
    (comparison.py:873-882), by the normal equations."""
    x, t = sim.reshape(-1), target.reshape(-1)
    A = torch.stack([x, torch.ones_like(x)], 1)
    coef = torch.linalg.solve(A.T @ A, A.T @ t)
    r = A @ coef - t
    return (r * r).sum()
