"""gw_detector_noalloc: the detector image for callers that cannot allocate
device memory when they need it (a loop that reserved its GPU memory budget
up front, or one where a cudaMalloc/cudaFree stall or failure mid-run is not
acceptable).  The test plays such a caller: it owns every device buffer and
passes plain device pointers through the C ABI, then checks the image
against the plan-based entry point gw_detector on two calls in a row.

This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-5  # same bar as the other detector parity tests


def _case():
    from giwaxsim_gb300 import forward as F
    rng = np.random.default_rng(11)
    n = 41
    q = np.linspace(-1.6, 1.6, n)
    iq = rng.uniform(0.1, 1.0, (n, n, n)) ** 4
    psis = np.linspace(0, 180, 9)
    phis = np.array([0.0, 25.0])
    thetas = np.array([0.0, 7.5])
    w = lambda a: np.ones_like(a) / len(a)
    plan = F.DetectorPlan(iq.shape, q, q, q, 48, 1.5, (90.0, 30.0, 0.0),
                          ("psi", "phi", "None"), psis, w(psis), phis, w(phis),
                          thetas, w(thetas), mirror=True)
    plan.close()  # only its host-side matrices and parameters are used
    return iq, plan


def test_noalloc_matches_plan_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    from giwaxsim_gb300 import _native as N
    iq, plan = _case()
    lib = N.lib()
    ctx = N.default_context(0)
    p = plan.params
    n_init = 0 if plan._init is None else len(plan._init)
    ref = np.empty((p.n_v, p.n_h))
    N.check(lib.gw_detector(ctx.handle, ctypes.byref(p), N.ptr(iq),
                            N.ptr(plan._h), N.ptr(plan._v), N.ptr(plan._init),
                            n_init, N.ptr(plan._nrot), N.ptr(plan._mats),
                            N.ptr(plan._w), plan.n_orient, N.ptr(ref)))

    dev = torch.device("cuda:0")
    iq32 = torch.tensor(iq, dtype=torch.float32, device=dev)
    h = torch.tensor(plan._h, device=dev)
    v = torch.tensor(plan._v, device=dev)
    init = torch.tensor(plan._init, device=dev)
    nrot = torch.tensor(plan._nrot, device=dev)
    mats = torch.tensor(plan._mats, device=dev)
    wts = torch.tensor(plan._w, device=dev)
    out = torch.empty((p.n_v, p.n_h), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        out.fill_(float("nan"))
        N.check(lib.gw_detector_noalloc(
            ctypes.byref(p), ctypes.c_void_p(iq32.data_ptr()),
            ctypes.c_void_p(h.data_ptr()), ctypes.c_void_p(v.data_ptr()),
            ctypes.c_void_p(init.data_ptr()), n_init,
            ctypes.c_void_p(nrot.data_ptr()), ctypes.c_void_p(mats.data_ptr()),
            ctypes.c_void_p(wts.data_ptr()), plan.n_orient,
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)))
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert np.all(np.isfinite(got)), call
        assert err <= RTOL, (call, err)


def test_noalloc_rejects_images_beyond_its_scratch():
    from giwaxsim_gb300 import _native as N
    _, plan = _case()
    p = N.DetectorParams.from_buffer_copy(plan.params)
    p.n_h = p.n_v = 1025
    dummy = ctypes.c_void_p(1)
    st = N.lib().gw_detector_noalloc(ctypes.byref(p), dummy, dummy, dummy,
                                     None, 0, dummy, None, dummy, 1, dummy,
                                     None)
    assert st == N.GW_ERR_ARG
    assert "1048576" in N.last_error()
