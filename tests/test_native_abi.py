"""The C ABI library: it loads, exports every symbol the public header
declares, and its host-only helpers (no GPU needed) match the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from oracle import giwaxs_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "giwaxs_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gw_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(N.LIB_PATH):
        from giwaxsim_gb300 import build
        build.build()
    return N.lib()


def test_header_and_binding_agree():
    assert header_functions() == sorted(N.EXPORTS)


def test_library_exports_every_header_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.gw_version() >= 1
    assert lib.gw_status_string(5) == b"GW_ERR_BOUNDS"


def test_missing_library_fails_loudly(monkeypatch):
    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setattr(N, "LIB_PATH", "/nonexistent/libgiwaxs_gb300.so")
    with pytest.raises(N.NativeLibraryMissing):
        N.lib()


def test_rotate_points_matches_blas_order(lib):
    from tests.conftest import golden
    d = golden("golden_rotation.npz")
    for phi, ref in zip(d["phis"], d["rot"]):
        pr = np.radians(phi)
        R = np.array([[np.cos(pr), -np.sin(pr), 0], [np.sin(pr), np.cos(pr), 0],
                      [0, 0, 1]])
        assert np.array_equal(N.rotate_points(R, d["coords"]), ref)


def test_collapse_base_uses_scalar_pow(lib):
    rng = np.random.default_rng(5)
    ver = rng.uniform(10, 300, 5000)
    ct = np.cos(np.deg2rad(rng.uniform(0, 90, 5000)))
    ref = np.array([np.sqrt(v ** 2 - (v * c) ** 2) for v, c in
                    zip(map(np.float64, ver), map(np.float64, ct))])
    assert np.array_equal(N.collapse_base(ver, ct), ref)


def test_error_reporting_without_gpu(lib):
    out = ctypes.c_void_p()
    st = lib.gw_voxel_plan_create(None, None, None, 0, None, 0,
                                  ctypes.byref(out))
    assert st == N.GW_ERR_ARG
    assert "null argument" in N.last_error()
    with pytest.raises(N.GwError, match="GW_ERR_ARG"):
        N.check(st)


def test_noalloc_limits_checked_before_any_device_call(lib):
    """The allocation-free detector call rejects null pointers and images
    beyond its fixed scratch (1024 x 1024 pixels) on the host, before it
    touches a device: the pointers below are never dereferenced."""
    p = N.DetectorParams()
    p.n_h, p.n_v = 1025, 1024
    p.iq_shape[:] = [4, 4, 4]
    p.dq = 0.1
    fake = ctypes.c_void_p(16)
    n_rot = ctypes.c_void_p(32)
    args = [ctypes.byref(p), fake, fake, fake, None, 0, n_rot, fake, fake, 1,
            fake, None]
    assert lib.gw_detector_noalloc(*args) == N.GW_ERR_ARG
    assert "1048576" in N.last_error()
    args[1] = None
    assert lib.gw_detector_noalloc(*args) == N.GW_ERR_ARG
    assert "null argument" in N.last_error()


def test_product_imports_no_oracle_or_tests():
    """The package never imports the oracle or the tests: the oracle is only
    the checker, never a fallback of the product path."""
    import ast
    import pathlib
    root = pathlib.Path(__file__).resolve().parents[1] / "giwaxsim_gb300"
    for path in root.rglob("*.py"):
        tree = ast.parse(path.read_text(), str(path))
        for node in ast.walk(tree):
            names = []
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom) and node.module:
                names = [node.module]
            for n in names:
                top = n.split(".")[0]
                assert top not in ("oracle", "tests"), (path, n)
