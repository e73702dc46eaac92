"""The dense float64 torch reference of the differentiable model, pinned on
CPU: its nearest-bin image equals the numpy oracle's (itself pinned to the
reference), its autograd gradient equals central differences of its own
forward, and the closed-form scale/offset misfit equals numpy's lstsq."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import giwaxs_oracle as O  # noqa: E402
from tests.grad_reference import DenseModel, misfit  # noqa: E402
from giwaxsim_gb300 import workloads as W  # noqa: E402


def small_case(seed=0, size=(9.0, 9.0, 9.0), disp=0.05):
    rng = np.random.default_rng(seed)
    xyz, _ = W.silicon_slab(size, rng, disp_sigma=disp)
    f = np.full(len(xyz), 14.0 + 0.3j)
    occ = rng.uniform(0.8, 1.0, len(xyz))
    return xyz, f, occ


GEOM = dict(r=0.3, dq=0.12, max_q=2.0)
PHIS = np.linspace(0.0, 180.0, 12, endpoint=False)


def model(deposit, f):
    return DenseModel(f, GEOM["r"], GEOM["dq"], GEOM["max_q"], PHIS, 48,
                      (0, 0, 0), ("None",) * 3, np.linspace(0, 90, 7),
                      deposit=deposit)


@pytest.mark.parametrize("sigma", [0.0, 1.5])
def test_dense_nearest_matches_oracle(sigma):
    xyz, f, occ = small_case()
    m = model("nearest", f)
    img = m.image(torch.as_tensor(xyz), torch.as_tensor(occ),
                  torch.tensor(sigma, dtype=torch.float64)).numpy()
    fo = f * occ
    out = O.voxelgrid([(xyz, fo)], GEOM["r"], GEOM["dq"], GEOM["max_q"],
                      phis=PHIS, smooth=sigma)
    q = out["qx"]
    det, _, _ = O.detector(out["iq"], q, q, q, 48, GEOM["max_q"], (0, 0, 0),
                           ("None",) * 3, np.linspace(0, 90, 7), None, [0.0],
                           None, [0.0], None, mirror=True)
    rel = np.linalg.norm(img - det) / np.linalg.norm(det)
    assert rel < 1e-12, rel


@pytest.mark.parametrize("deposit", ["nearest", "bilinear"])
def test_dense_gradient_matches_central_differences(deposit):
    xyz, f, occ = small_case(seed=1)
    m = model(deposit, f)
    X, Oc, S = (torch.as_tensor(xyz), torch.as_tensor(occ),
                torch.tensor(1.5, dtype=torch.float64))
    rng = np.random.default_rng(5)
    target = torch.as_tensor(m.image(X, Oc * 0.95, S).numpy()
                             * rng.uniform(0.9, 1.1, (48, 48)))
    loss_fn = lambda img: misfit(img, target)  # noqa: E731
    _, g_occ, g_sig, g_xyz = m.gradient(loss_fn, X, Oc, S, chunk=5)

    def L(X_, O_, S_):
        return float(loss_fn(m.image(X_, O_, S_)))

    h = 1e-4
    for a in rng.choice(len(occ), 4, replace=False):
        d = torch.zeros_like(Oc)
        d[a] = h
        fd = (L(X, Oc + d, S) - L(X, Oc - d, S)) / (2 * h)
        assert abs(fd - float(g_occ[a])) <= 1e-5 * abs(fd) + 1e-9 * float(g_occ.abs().max())
    fd = (L(X, Oc, S + h) - L(X, Oc, S - h)) / (2 * h)
    assert abs(fd - float(g_sig)) <= 1e-5 * abs(fd) + 1e-12
    if deposit == "bilinear":
        # interior atoms, small steps that cross no cell boundary
        for a in rng.choice(len(occ), 3, replace=False):
            for ax in range(3):
                d = torch.zeros_like(X)
                d[a, ax] = 1e-5
                fd = (L(X + d, Oc, S) - L(X - d, Oc, S)) / 2e-5
                assert abs(fd - float(g_xyz[a, ax])) <= (
                    1e-4 * abs(fd) + 1e-7 * float(g_xyz.abs().max()))


def test_misfit_matches_lstsq():
    rng = np.random.default_rng(2)
    x = rng.random((20, 20))
    t = 3.0 * x + 0.5 + rng.normal(0, 0.01, x.shape)
    A = np.vstack([x.ravel(), np.ones(x.size)]).T
    (s, b), *_ = np.linalg.lstsq(A, t.ravel(), rcond=None)
    ref = np.sum((s * x + b - t) ** 2)
    got = float(misfit(torch.as_tensor(x), torch.as_tensor(t)))
    assert abs(got - ref) <= 1e-9 * ref
    from giwaxsim_gb300.autograd import scale_offset_misfit
    got2, s2, b2 = scale_offset_misfit(torch.as_tensor(x), torch.as_tensor(t))
    assert abs(float(got2) - ref) <= 1e-9 * ref
    assert abs(float(s2) - s) < 1e-9 and abs(float(b2) - b) < 1e-9
