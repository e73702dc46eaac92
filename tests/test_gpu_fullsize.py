"""The timed configuration checked in full: si-100A (diamond Si, 100 A cube,
~50 k atoms, g = 1257, 360 phi slices, fill_bkg, smooth = 2) through the
batched voxel stage, and its 1000 px detector image over 91 orientations
(init psi = 90, psi 0..90), against the float64 oracle over every slice and
every orientation (tools/comparison.py:673-870).  Counts bit-exact; I(q)
and the image within 1e-5 normwise relative L2.  The oracle runs threaded
over slices and orientations (a few seconds on the GPU machine's host)."""
import os

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from oracle import giwaxs_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
NAME = "si-100A"


@pytest.fixture(scope="module")
def case():
    w = W.WORKLOADS[NAME]
    (xyz, el, wt), = W.structures(NAME)
    phis = W.phis_linspace(w["n_phi"])
    fv = F.element_f_values(el, w["energy"])
    workers = min(32, (os.cpu_count() or 1) + 4)
    ref = O.voxelgrid_crop_threaded(xyz, fv, w["r"], w["dq"], w["max_q"], phis,
                                    w["fill_bkg"], w["smooth"], workers)
    a, b, n = w["psis"]
    psis = np.linspace(a, b, n)
    one = np.array([0.0])
    det_args = (w["num_pixels"], w["max_q"]) + w["init"] + (
        psis, np.ones(n) / n, one, np.ones(1), one, np.ones(1))
    dref = O.detector_threaded(ref["iq"], ref["q"], ref["q"], ref["q"],
                               *det_args, True, workers)[0]
    return w, xyz, fv, phis, ref, dref, det_args


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("tune", [False, True])
def test_si_100A_all_slices_and_detector_vs_oracle(case, tune):
    w, xyz, fv, phis, ref, dref, det_args = case
    ctx = N.default_context(0)
    geom = F.VoxelGeometry(w["r"], w["dq"], w["max_q"])
    plan = F.VoxelPlan(geom, [(xyz, fv, None)], phis=phis, fill_bkg=w["fill_bkg"],
                       smooth=w["smooth"], tune=tune, ctx=ctx)
    plan.set_atoms()
    plan.execute()
    ctx.synchronize()
    plan.capture_graph()
    plan.execute()                      # the graph replay the bench times
    ctx.synchronize()
    assert np.array_equal(plan.counts(), ref["count"])
    e_iq = rel(plan.iq(), ref["iq"])
    assert e_iq <= TOL, e_iq
    q = geom.q_crop
    assert np.array_equal(q, ref["q"])
    det = F.DetectorPlan((plan.Qc,) * 3, q, q, q, *det_args, mirror=True,
                         ctx=ctx)
    det.set_iq_device32(plan.device_iq32())
    det.execute()
    img = det.result()
    e_det = rel(img, dref)
    assert e_det <= TOL, e_det
    det.close()
    plan.close()
