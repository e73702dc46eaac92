"""The conversion helpers the hot kernels use instead of hardware
conversions (floor to int by magic-number rounding, float <-> double by
IEEE 754 bit manipulation) against numpy, bit for bit, and the float32
I(q) the finalize writes against the float64 I(q) rounded."""
import ctypes

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _convert(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    f32 = np.empty(n, np.float32)
    f64 = np.empty(n)
    fl = np.empty(n, np.int32)
    ok = np.empty(n, np.int32)
    N.check(N.lib().gw_debug_convert(N.default_context().handle, N.ptr(x), n,
                                     N.ptr(f32), N.ptr(f64), N.ptr(fl), N.ptr(ok)))
    return f32, f64, fl, ok


def test_conversions_bit_exact():
    rng = np.random.default_rng(0)
    one = np.float64(1.0)
    eps = np.finfo(np.float32).eps
    specials = [0.0, -0.0, 1.0, -1.0, 0.5, 1.5, 2.5, -2.5, 1e-40, -1e-40,
                1e-45, 3.4028234663852886e38, 3.4028235677973366e38, 1e39,
                -1e39, np.inf, -np.inf, 1.0 + eps / 2, 1.0 + eps * 1.5,
                1.0 - eps / 4, 2097151.5, -2097151.5, 2097152.0, -2097152.0,
                1.1754943508222875e-38, 1.1754942106924411e-38, 123456.49999999999,
                np.nextafter(one, 2.0), np.nextafter(one, 0.0), 16777215.5]
    # doubles that sit exactly half-way between floats, and next to it
    mid = (np.float64(np.float32(1.3)) +
           np.float64(np.nextafter(np.float32(1.3), np.float32(2))) ) / 2
    specials += [mid, np.nextafter(mid, 0), np.nextafter(mid, 2), -mid]
    x = np.concatenate([np.array(specials), rng.normal(0, 1e3, 200000),
                        rng.uniform(-3e6, 3e6, 100000),
                        np.exp(rng.uniform(-200, 200, 100000)),
                        np.round(rng.uniform(-1e5, 1e5, 50000)),
                        np.round(rng.uniform(-1e5, 1e5, 50000)) + 0.5])
    f32, f64, fl, ok = _convert(x)
    ref32 = x.astype(np.float32)
    assert np.array_equal(f32.view(np.uint32), ref32.view(np.uint32))
    assert np.array_equal(f64.view(np.uint64), ref32.astype(np.float64).view(np.uint64))
    fin = np.abs(ref32) < 2097152.0
    assert np.array_equal(ok.astype(bool), fin)
    assert np.array_equal(fl[fin], np.floor(ref32[fin]).astype(np.int64))


def test_float32_iq_within_two_ulps_of_float64_iq():
    """The step's float32 I(q) (the detector's input) is computed in
    float32 from the float64 sum rounded to float, RN(RN(s) * f), so that
    the step does no float64 arithmetic; the float64 I(q) is s * f with one
    rounding.  The two differ by at most 1.5 float32 ulps (checked as 2 on
    the bit patterns, which are ordered like the values for positives), and
    are zero together."""
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    rng = np.random.default_rng(5)
    xyz, _ = W.graphite_slab((12.0, 11.0, 13.0), rng, disp_sigma=0.05)
    for fill, smooth in ((False, 0), (True, 1.5)):
        plan = F.VoxelPlan(geom, [(xyz, np.full(len(xyz), 6.0 + 0j), None)],
                           phis=np.linspace(0, 180, 30, endpoint=False),
                           fill_bkg=fill, smooth=smooth)
        plan.set_atoms()
        plan.execute()
        i64, i32 = plan.iq(), plan.iq32()
        r32 = i64.astype(np.float32)
        assert np.all(i32 >= 0) and np.array_equal(i32 == 0, r32 == 0)
        ulps = np.abs(i32.view(np.int32).astype(np.int64)
                      - r32.view(np.int32).astype(np.int64))
        assert ulps.max() <= 2, ulps.max()
        plan.close()
