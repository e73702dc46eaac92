"""The experimental-comparison step on the device against the reference's
own trim_sim_data / rebin_qmap_and_mask / optimize_scale_offset outputs
(tests/golden/golden_compare.npz): the rebinned map and mask bit for bit,
scale, offset and residuals to 1e-12 (normal equations on the device vs
numpy's lstsq)."""
import numpy as np
import pytest

from giwaxsim_gb300.tools import comparison
from tests.conftest import golden

pytestmark = pytest.mark.gpu


def test_rebin_drop_in_bit_exact():
    d = golden("golden_compare.npz")
    m, mk = comparison.rebin_qmap_and_mask(d["h_trim"], d["v_trim"], d["exp_img"],
                                           d["exp_qxy"], d["exp_qz"], d["mask"])
    assert np.array_equal(m, d["rebin_raw"], equal_nan=True)
    assert np.array_equal(mk, d["rebin_mask"])


def test_comparison_plan_vs_reference():
    d = golden("golden_compare.npz")
    c = comparison.Comparison(d["det_h"], d["det_v"], d["exp_img"], d["exp_qxy"],
                              d["exp_qz"], d["mask"])
    t, mk = c.target()
    assert np.array_equal(t, d["rebin_raw"], equal_nan=True)
    assert np.array_equal(mk, d["rebin_mask"])
    s, o, mis, n, res = c.evaluate(d["sim"], residual=True)
    assert n == int((d["rebin_mask"] == 0).sum())
    assert abs(s - d["scale"]) <= 1e-12 * abs(d["scale"])
    assert abs(o - d["offset"]) <= 1e-12 * max(abs(d["offset"]), 1.0)
    ref = d["residual"]
    assert np.abs(res - ref).max() <= 1e-12 * np.abs(d["rebin_raw"]).max()
    assert abs(mis - float((ref ** 2).sum())) <= 1e-9 * float((ref ** 2).sum())
    # misfit from the moments alone (no residual map) agrees; the moments'
    # float64 atomics add in scheduling order
    s2, o2, mis2, _ = c.evaluate(d["sim"])
    assert abs(s2 - s) <= 1e-13 * abs(s) and abs(o2 - o) <= 1e-13 * max(abs(o), 1.0)
    assert abs(mis2 - mis) <= 1e-8 * mis
    c.close()


def test_optimize_scale_offset_drop_in():
    rng = np.random.default_rng(0)
    sim = rng.uniform(0, 1, (20, 20))
    mask = (rng.uniform(0, 1, (20, 20)) > 0.8).astype(int)
    reb = 3.0 * sim + 0.25
    s, o = comparison.optimize_scale_offset(sim, reb, mask)
    assert abs(s - 3.0) < 1e-12 and abs(o - 0.25) < 1e-12
    d = golden("golden_compare.npz")
    reb = d["rebin_raw"].copy()
    reb[d["rebin_mask"] == 1] = 0
    s, o = comparison.optimize_scale_offset(d["sim_trim"], reb, d["rebin_mask"])
    assert abs(s - d["scale"]) <= 1e-12 * abs(d["scale"])
    assert abs(o - d["offset"]) <= 1e-12 * max(abs(d["offset"]), 1.0)
