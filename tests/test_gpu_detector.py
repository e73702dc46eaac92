"""GPU detector stage against the oracle and the reference fixtures.

Gathered voxel indices are compared bit-exact; images by normwise relative
L2 <= 1e-5 (float32 I(q) samples summed in float64)."""
import numpy as np
import pytest

from giwaxsim_gb300 import forward as F
from giwaxsim_gb300.tools import comparison
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def synthetic_iq(n=41, qmax=1.6, seed=0):
    rng = np.random.default_rng(seed)
    q = np.linspace(-qmax, qmax, n)
    iq = rng.uniform(0.1, 1.0, (n, n, n)) ** 4
    return iq, q


CASES = [
    # (init vals, init axes, psis, phis, thetas, mirror, pixels)
    ((0, 0, 0), ("None",) * 3, np.linspace(0, 180, 13), [0.0], [0.0], True, 31),
    ((90.0, 0, 0), ("psi", "None", "None"), np.linspace(0, 90, 10), [0.0],
     [0.0], True, 40),
    ((90.0, 30.0, 10.0), ("psi", "phi", "theta"), np.linspace(0, 180, 7),
     [0.0, 20.0], [0.0, 5.0], False, 25),
    ((0, 45.0, 0), ("None", "phi", "None"), np.linspace(10, 170, 5),
     [0.0, 33.0, 71.0], [12.0], True, 24),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_detector_vs_oracle(case):
    init, axs, psis, phis, thetas, mirror, npx = CASES[case]
    iq, q = synthetic_iq()
    ref, h, v = O.detector(iq, q, q, q, npx, 1.5, init, axs, psis, None,
                           np.asarray(phis), None, np.asarray(thetas), None,
                           mirror=mirror)
    got, gh, gv = comparison.detectormaker_fitting(
        iq, q, q, q, npx, 1.5, init, axs, psis, None, np.asarray(phis), None,
        np.asarray(thetas), None, mirror=mirror)
    assert np.array_equal(gh, h) and np.array_equal(gv, v)
    assert rel_l2(got, ref) <= RTOL


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_gather_indices_bit_exact(case, exact):
    """The voxel each pixel gathers, per orientation, equals the oracle's
    (the fast path's float32 decisions plus its exact replays, and the
    all-exact path)."""
    init, axs, psis, phis, thetas, mirror, npx = CASES[case]
    iq, q = synthetic_iq()
    psis, phis, thetas = map(np.asarray, (psis, phis, thetas))
    w = lambda a: np.ones_like(a) / len(a)
    plan = F.DetectorPlan(iq.shape, q, q, q, npx, 1.5, init, axs, psis,
                          w(psis), phis, w(phis), thetas, w(thetas), mirror,
                          exact=exact)
    plan.set_iq(iq)
    x0, y0, z0, _, _ = O.init_detector(npx, 1.5, init, axs)
    o = 0
    for ps in psis:
        for ph in phis:
            for th in thetas:
                x, y, z = O.rotate_psi_phi_theta(x0, y0, z0, ps, ph, th)
                iy, ix, iz = O.intersect_indices(iq.shape, q, q, q, x, y, z)
                ref = (iy * iq.shape[1] + ix) * iq.shape[2] + iz
                assert np.array_equal(plan.debug_indices(o), ref), (ps, ph, th)
                o += 1


def test_reference_fixture_detector():
    v = golden("golden_voxel.npz")
    d = golden("golden_detector.npz")
    iq, qx, qy, qz = v["iq_plain"], v["qx"], v["qy"], v["qz"]
    det, h, vv = comparison.detectormaker_fitting(
        iq, qx, qy, qz, 21, 1.2, (90.0, 30.0, 10.0), ("psi", "phi", "theta"),
        np.linspace(0, 180, 7), None, np.array([0.0, 20.0]), None,
        np.array([0.0, 5.0]), None, mirror=True)
    assert rel_l2(det, d["det_sum"]) <= RTOL
    det2, _, _ = comparison.detectormaker_fitting(
        iq, qx, qy, qz, 16, 1.2, (0.0, 0.0, 0.0), ("None",) * 3,
        np.linspace(0, 90, 10), None, np.array([0.0]), None, np.array([0.0]),
        None, mirror=True)
    assert rel_l2(det2, d["det_sum2"]) <= RTOL


def test_kahan32_accumulation():
    iq, q = synthetic_iq(seed=3)
    args = (iq, q, q, q, 48, 1.5, (0, 0, 0), ("None",) * 3,
            np.linspace(0, 180, 181), None, np.array([0.0]), None,
            np.array([0.0]), None)
    ref, _, _ = O.detector(*args, mirror=True)
    got, _, _ = comparison.detectormaker_fitting(*args, mirror=True,
                                                 accum="kahan32")
    assert rel_l2(got, ref) <= RTOL


def test_weights_and_errors(tmp_path):
    iq, q = synthetic_iq()
    psis = np.linspace(0, 90, 4)
    wpath = tmp_path / "w.npy"
    np.save(wpath, np.array([0.1, 0.2, 0.3, 0.4]))
    ref, _, _ = O.detector(iq, q, q, q, 20, 1.5, (0, 0, 0), ("None",) * 3,
                           psis, np.load(wpath), np.array([0.0]), None,
                           np.array([0.0]), None, mirror=True)
    got, _, _ = comparison.detectormaker_fitting(
        iq, q, q, q, 20, 1.5, (0, 0, 0), ("None",) * 3, psis, str(wpath),
        np.array([0.0]), None, np.array([0.0]), None, mirror=True)
    assert rel_l2(got, ref) <= RTOL
    np.save(wpath, np.array([0.1, 0.2, 0.3]))
    with pytest.raises(AssertionError, match="psi weights length"):
        comparison.detectormaker_fitting(
            iq, q, q, q, 20, 1.5, (0, 0, 0), ("None",) * 3, psis, str(wpath),
            np.array([0.0]), None, np.array([0.0]), None)


@pytest.mark.parametrize("cap", [None, "7"])
def test_fast_path_matches_exact_path(cap, monkeypatch):
    """Fast image == all-exact image to rounding (different summation order);
    cap=7 forces the worklist to overflow so the in-kernel exact branch runs."""
    if cap:
        monkeypatch.setenv("GW_DET_WORKLIST_CAP", cap)
    iq, q = synthetic_iq(seed=5)
    init, axs, psis, phis, thetas, mirror, npx = CASES[2]
    args = (iq, q, q, q, 64, 1.5, init, axs, psis, None, np.asarray(phis),
            None, np.asarray(thetas), None)
    fast, _, _ = comparison.detectormaker_fitting(*args, mirror=mirror)
    exact, _, _ = comparison.detectormaker_fitting(*args, mirror=mirror,
                                                   exact=True)
    ref, _, _ = O.detector(*args, mirror=mirror)
    assert rel_l2(fast, exact) <= 1e-6
    assert rel_l2(fast, ref) <= RTOL


def test_large_detector_vs_oracle():
    """500 px, 91 orientations on a 203^3 grid (graphite-50A detector sizes)."""
    iq, q = synthetic_iq(n=203, qmax=3.03, seed=7)
    psis = np.linspace(0, 180, 91)
    args = (iq, q, q, q, 500, 3.0, (0, 0, 0), ("None",) * 3, psis, None,
            np.array([0.0]), None, np.array([0.0]), None)
    got, _, _ = comparison.detectormaker_fitting(*args, mirror=True)
    ref, _, _ = O.detector(*args, mirror=True)
    assert rel_l2(got, ref) <= RTOL


@pytest.mark.parametrize("n,npx,cap", [(41, 31, None), (41, 40, "7"),
                                       (203, 500, None), (260, 300, None)])
def test_plane_gather_bit_identical(n, npx, cap, monkeypatch):
    """Orientations that keep x = 0 (rotations about the detector normal)
    take the plane gather -- from shared memory (plane <= 200 KB) or global
    memory (260^2 floats) -- and gather the same samples as the general fast
    path: the images agree to the order of the float64 atomic adds of the
    exactly replayed samples (1e-12).  cap=7 overflows the worklist into the
    in-kernel exact branch; which samples overflow depends on push order, and
    those go into the float32 partial sums (1e-7)."""
    if cap:
        monkeypatch.setenv("GW_DET_WORKLIST_CAP", cap)
    iq, q = synthetic_iq(n=n, qmax=1.5 * (n - 1) / 40, seed=3)
    psis = np.linspace(0, 180, 37)
    one = np.array([0.0])
    for init, axs in (((0, 0, 0), ("None",) * 3),
                      ((90.0, 0, 0), ("psi", "None", "None"))):
        imgs, launches = [], []
        for plane in (True, False):
            p = F.DetectorPlan(iq.shape, q, q, q, npx, q[-1], init, axs, psis,
                               np.ones_like(psis) / len(psis), one, one + 1,
                               one, one + 1, mirror=True, plane=plane)
            p.set_iq(iq)
            c0 = p.ctx.launch_count()
            p.execute()
            launches.append(p.ctx.launch_count() - c0)
            imgs.append(p.result())
            p.close()
        assert launches[0] == launches[1] + 1  # + the plane copy
        assert rel_l2(imgs[0], imgs[1]) <= (1e-7 if cap else 1e-12)
