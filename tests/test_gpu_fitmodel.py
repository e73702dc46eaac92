"""shift_peak on the device and the fullfit_model drop-in
(fit_slabsize.py:19-46) against the oracle."""
import os

import numpy as np
import pytest

from giwaxsim_gb300.fit import fullfit_model
from giwaxsim_gb300.tools import comparison
from giwaxsim_gb300.tools.utilities import calc_real_space_abc, load_xyz
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["pad", "nopad"])
def test_device_shift_peak_vs_reference(name):
    d = golden("golden_shift.npz")
    out = comparison.shift_peak(d["img"].copy(), d["det_h"], d["det_v"],
                                float(d[name + "_pw"]), tuple(d[name + "_pr"]))
    ref = d[name + "_out"]
    assert np.abs(out - ref).max() <= 1e-14 * np.abs(ref).max()


def test_fullfit_model_vs_oracle(tmp_path):
    cellp = (2.46, 2.46, 6.70, 90.0, 90.0, 120.0)
    vecs = np.array(calc_real_space_abc(*cellp))
    frac = np.array([[0, 0, 0.25], [0, 0, 0.75], [1 / 3, 2 / 3, 0.25],
                     [2 / 3, 1 / 3, 0.75]])
    path = os.path.join(str(tmp_path), "graphite.xyz")
    with open(path, "w") as fh:
        fh.write("4\ncell\n")
        for x, y, z in frac @ vecs:
            fh.write("C %.17g %.17g %.17g\n" % (x, y, z))
    cell_xyz, cell_el = load_xyz(path)
    r, dq, max_q, num_pixels = 0.5, 0.1, 1.6, 48
    psis = np.linspace(0, 180, 7)
    det_phis, thetas = np.array([0.0]), np.array([0.0])
    init_vals, init_axs = (0, 0, 0), ("None", "None", "None")
    # the trimmed grid of the experiment's range, and a synthetic rebinned map
    h = np.linspace(-max_q, max_q, num_pixels)
    exp_qxy, exp_qz = np.linspace(0.05, 1.5, 40), np.linspace(0.0, 1.5, 35)
    hm = (h >= exp_qxy.min()) & (h <= exp_qxy.max())
    vm = (h >= exp_qz.min()) & (h <= exp_qz.max())
    gh, gv = np.meshgrid(h[hm], h[vm])
    rng = np.random.default_rng(4)
    rebin_map = np.exp(-((np.hypot(gh, gv) - 1.2) / 0.1) ** 2) + 0.02 * rng.random(gh.shape)
    rebin_mask = (rng.random(gh.shape) < 0.1).astype(int)
    rebin_map[rebin_mask == 1] = 0
    fixed = ((path,) + cellp,
             (r, dq, max_q, 10000.0, False, 0),
             (num_pixels, init_vals, init_axs, psis, None, det_phis, None,
              thetas, None),
             (rebin_map, rebin_mask, exp_qxy, exp_qz, 0.05, (0.6, 1.4)))
    for size in ((26.0, 27.0, 28.0), (30.0, 27.0, 28.0)):
        params = {"x_size": size[0], "y_size": size[1], "z_size": size[2]}
        got = fullfit_model(params, *fixed)
        ref, _, _ = O.fullfit_residuals(
            cell_xyz, cell_el, vecs, size, r, dq, max_q, {"C": 6.0 + 0j},
            num_pixels, init_vals, init_axs, psis, None, det_phis, None,
            thetas, None, rebin_map, rebin_mask, exp_qxy, exp_qz, 0.05,
            (0.6, 1.4))
        assert got.shape == ref.shape
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(rebin_map)
        assert np.all(got[rebin_mask.ravel() == 1] == 0.0)
