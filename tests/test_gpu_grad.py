"""Adjoint kernels against the dense float64 torch reference and float64
central differences.

  * small Si slab: GPU image vs dense image (nearest and bilinear deposit,
    with and without smoothing), GPU gradient vs dense autograd gradient;
  * si-60A-occ (60 A Si cube, g=512, 180 phis, 512 px detector, psi 0..90,
    sigma 1.5, bilinear deposit, checkpoint interval 16): image and full
    gradient vs the dense reference, and 32 random parameters (occupancies,
    sigma, coordinates) vs central differences with h = 1e-3 of the dense
    float64 forward.

Tolerances: images 1e-5 normwise; gradients 1e-4 (normwise per parameter
group against the dense gradient; against central differences, normwise
over the 32 parameters and per parameter relative to the largest).
Coordinates are perturbed by 0.02 A so that no two atoms tie for a minimum
or maximum (the shift to the minimum and the slab bounds then have one
owner).  Coordinate differences use atoms that stay clear of cell
boundaries (3h/r) in every slice: the bilinear deposit is piecewise linear
and a step across a boundary would average two slopes.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import giwaxs_oracle as O  # noqa: E402
from tests.grad_reference import DenseModel, misfit  # noqa: E402
from giwaxsim_gb300 import workloads as W  # noqa: E402
from giwaxsim_gb300.autograd import (DetectorModel, detector_image,  # noqa: E402
                                     scale_offset_misfit)

pytestmark = pytest.mark.gpu


def _dev():
    return "cuda" if torch.cuda.is_available() else "cpu"


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def models(xyz, energy, r, dq, max_q, phis, npix, psis, deposit, k=16):
    el = np.full(len(xyz), "Si")
    gm = DetectorModel(el, energy, r, dq, max_q, npix, psis=psis, phis=phis,
                       deposit=deposit, checkpoint_every=k, mirror=True)
    dm = DenseModel(gm.f_el, r, dq, max_q, phis, npix, (0, 0, 0),
                    ("None",) * 3, psis, deposit=deposit, device=_dev())
    return gm, dm


def gpu_grad(gm, xyz, occ, sigma, target, want_xyz):
    o = torch.tensor(occ, dtype=torch.float64, requires_grad=True)
    s = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    x = torch.tensor(xyz, dtype=torch.float64, requires_grad=want_xyz)
    img = detector_image(gm, o, s, x)
    loss, _, _ = scale_offset_misfit(img, torch.as_tensor(target))
    loss.backward()
    return (float(loss), o.grad.numpy(), float(s.grad),
            x.grad.numpy() if want_xyz else None, img.detach().numpy())


def small_slab(seed):
    rng = np.random.default_rng(seed)
    xyz, _ = W.silicon_slab((9.0, 9.0, 9.0), rng, disp_sigma=0.05)
    return xyz, rng


SMALL = dict(energy=11000.0, r=0.3, dq=0.12, max_q=2.0,
             phis=np.linspace(0.0, 180.0, 12, endpoint=False), npix=48,
             psis=np.linspace(0.0, 90.0, 7))


@pytest.mark.parametrize("deposit,sigma", [("nearest", 0.0), ("nearest", 1.5),
                                           ("bilinear", 0.0), ("bilinear", 1.5)])
def test_small_image_and_gradient(deposit, sigma):
    xyz, rng = small_slab(3)
    gm, dm = models(xyz, SMALL["energy"], SMALL["r"], SMALL["dq"],
                    SMALL["max_q"], SMALL["phis"], SMALL["npix"],
                    SMALL["psis"], deposit, k=5)
    hidden = rng.uniform(0.8, 1.0, len(xyz))
    dev = _dev()
    X = torch.as_tensor(xyz, device=dev)
    target = dm.image(X, torch.as_tensor(hidden, device=dev),
                      torch.tensor(sigma, dtype=torch.float64, device=dev))
    occ0 = np.full(len(xyz), 0.9)
    ref_img = dm.image(X, torch.as_tensor(occ0, device=dev),
                       torch.tensor(sigma, dtype=torch.float64, device=dev)).cpu().numpy()
    loss, g_occ, g_sig, g_xyz, img = gpu_grad(gm, xyz, occ0, sigma,
                                              target.cpu().numpy(),
                                              deposit == "bilinear")
    assert rel(img, ref_img) < 1e-5
    tgt = target
    _, r_occ, r_sig, r_xyz = dm.gradient(lambda im: misfit(im, tgt), X,
                                         torch.as_tensor(occ0, device=dev),
                                         torch.tensor(sigma, dtype=torch.float64,
                                                      device=dev), chunk=5)
    assert rel(g_occ, r_occ.cpu().numpy()) < 1e-4
    if sigma > 0:
        assert abs(g_sig - float(r_sig)) <= 1e-4 * abs(float(r_sig))
    else:
        assert g_sig == 0.0
    if deposit == "bilinear":
        assert rel(g_xyz, r_xyz.cpu().numpy()) < 1e-4
    gm.close()


def clean_atoms(xyz, phis, r, h):
    """Atoms whose cell fractions stay more than 3h/r from a boundary in
    every slice and which own no minimum/maximum."""
    margin = 3.0 * h / r
    ok = np.ones(len(xyz), bool)
    for phi in phis:
        y = O.rotate_coords_z(xyz, phi)[:, 1]
        u = (y - y.min()) / r
        fr = u - np.floor(u)
        ok &= (fr > margin) & (fr < 1 - margin)
        ok[np.argmin(y)] = False
    v = (xyz[:, 2] - xyz[:, 2].min()) / r
    fr = v - np.floor(v)
    ok &= (fr > margin) & (fr < 1 - margin)
    for ax in range(3):
        ok[np.argmin(xyz[:, ax])] = False
        ok[np.argmax(xyz[:, ax])] = False
    return np.where(ok)[0]


def test_si60_occupancy_sigma_coordinates_gradient():
    w = W.WORKLOADS["si-60A-occ"]
    (xyz, _, hidden), = W.structures("si-60A-occ")
    rng = np.random.default_rng(11)
    xyz = xyz + rng.normal(0.0, 0.02, xyz.shape)
    phis = W.phis_linspace(w["n_phi"])
    psis = np.linspace(*w["psis"])
    gm, dm = models(xyz, w["energy"], w["r"], w["dq"], w["max_q"], phis,
                    w["num_pixels"], psis, "bilinear", k=16)
    assert gm.geom.grid_size == 512
    dev = _dev()
    X = torch.as_tensor(xyz, device=dev)
    S0 = torch.tensor(1.5, dtype=torch.float64, device=dev)
    target = dm.image(X, torch.as_tensor(hidden, device=dev), S0)
    # start of a fit: full occupancy, a smoothing guess, coordinates off by
    # 0.05 A (an unrelaxed model).  sigma stays clear of the points where
    # the plateau bounds ceil(lo + sigma) (integer sigma) or the kernel
    # radius int(4 sigma + 0.5) jump.
    occ0 = np.full(len(xyz), 1.0)
    sig0 = 1.2
    xyz = xyz + rng.normal(0.0, 0.05, xyz.shape)
    X = torch.as_tensor(xyz, device=dev)
    loss, g_occ, g_sig, g_xyz, img = gpu_grad(gm, xyz, occ0, sig0,
                                              target.cpu().numpy(), True)
    O0 = torch.as_tensor(occ0, device=dev)
    S = torch.tensor(sig0, dtype=torch.float64, device=dev)
    ref_img = dm.image(X, O0, S)
    loss_fn = lambda im: misfit(im, target)  # noqa: E731
    r_loss, r_occ, r_sig, r_xyz = dm.gradient(loss_fn, X, O0, S, chunk=16)
    m = dict(image=rel(img, ref_img.cpu().numpy()),
             # |residual after the scale/offset fit| / |image|: the misfit's
             # relative error is the image's divided by this
             fit_residual=float(np.sqrt(r_loss)) / float(torch.linalg.norm(target)),
             loss=abs(loss - r_loss) / r_loss,
             occ=rel(g_occ, r_occ.cpu().numpy()),
             sigma=abs(g_sig - float(r_sig)) / abs(float(r_sig)),
             xyz=rel(g_xyz, r_xyz.cpu().numpy()))
    print("si-60A-occ vs dense float64:", m)
    assert m["image"] < 1e-5
    assert m["occ"] < 1e-4 and m["sigma"] < 1e-4 and m["xyz"] < 1e-4, m

    # 32 random parameters against float64 central differences, h = 1e-3
    h = 1e-3

    def L(X_, O_, S_):
        return float(loss_fn(dm.image(X_, O_, S_)))

    pick_occ = rng.choice(len(xyz), 15, replace=False)
    pick_at = rng.choice(clean_atoms(xyz, phis, w["r"], h), 16, replace=False)
    pick_ax = rng.integers(0, 3, 16)
    fd, gg = [], []
    for a in pick_occ:
        d = torch.zeros_like(O0)
        d[a] = h
        fd.append((L(X, O0 + d, S) - L(X, O0 - d, S)) / (2 * h))
        gg.append(g_occ[a])
    fd.append((L(X, O0, S + h) - L(X, O0, S - h)) / (2 * h))
    gg.append(g_sig)
    for a, ax in zip(pick_at, pick_ax):
        d = torch.zeros_like(X)
        d[a, ax] = h
        fd.append((L(X + d, O0, S) - L(X - d, O0, S)) / (2 * h))
        gg.append(g_xyz[a, ax])
    fd, gg = np.array(fd), np.array(gg)
    assert len(fd) == 32
    print("si-60A-occ vs central differences: normwise %.3g, max %.3g of max"
          % (rel(gg, fd), np.abs(gg - fd).max() / np.abs(fd).max()))
    assert rel(gg, fd) < 1e-4, (rel(gg, fd), np.abs(gg - fd).max())
    assert np.abs(gg - fd).max() <= 1e-4 * np.abs(fd).max()
    gm.close()
