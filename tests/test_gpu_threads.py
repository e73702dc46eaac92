"""Drop-in calls from several threads, as the reference's drivers make them
from a thread pool (comparison.py:759-763 for the slices, :850-853 for the
orientations): each thread works on its own context, and the threaded
results equal the serial ones."""
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import comparison as C
from giwaxsim_gb300.tools import detector as D
from giwaxsim_gb300.tools import utilities as U
from giwaxsim_gb300.tools import voxelgrids as V
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def shared(shape):
    m = U.create_shared_array(shape)
    np.ndarray(shape, dtype=np.float64, buffer=m.buf)[:] = 0
    return m


def read(m, shape):
    return np.ndarray(shape, dtype=np.float64, buffer=m.buf).copy()


def free(*ms):
    for m in ms:
        m.close()
        m.unlink()


def test_threaded_slice_workers_sum_like_serial():
    """rotate_project_fft_coords from a pool of 4 threads into one pair of
    named grids: counts equal the serial run's, sums up to the order of
    the additions, and both equal the reference fixture."""
    d = golden("golden_slices.npz")
    xyz, q, g, r = d["coords"], d["q"], int(d["g"]), float(d["r"])
    fv = np.full(len(xyz), 6.0 + 0j)
    xb, yb, zb, avg = O.structure_constants(xyz, fv, r)
    shape = (len(q),) * 3
    phis = list(d["phis"]) * 3          # more tasks than threads
    out = {}
    for name, workers in (("serial", 0), ("threads", 4)):
        s, c = shared(shape), shared(shape)
        try:
            args = [(xyz, fv, phi, g, r, avg, xb, yb, zb, True, 1, q, q, q,
                     s.name, c.name) for phi in phis]
            if workers:
                with ThreadPoolExecutor(max_workers=workers) as pool:
                    list(pool.map(V.rotate_project_fft_coords, args))
            else:
                for a in args:
                    V.rotate_project_fft_coords(a)
            out[name] = read(s, shape), read(c, shape)
        finally:
            free(s, c)
    (s1, c1), (s4, c4) = out["serial"], out["threads"]
    assert np.array_equal(c4, c1)
    assert np.array_equal(c1, 3 * d["count_fillsmooth"])
    assert rel_l2(s4, s1) <= 1e-12
    assert rel_l2(s1, 3 * d["sum_fillsmooth"]) <= 1e-5


def test_threaded_orientation_workers_sum_like_serial():
    """generate_detector_ints from a pool of 4 threads into one named image
    equals the serial sum."""
    v = golden("golden_voxel.npz")
    iq, qx, qy, qz = v["iq_plain"], v["qx"], v["qy"], v["qz"]
    x0, y0, z0, _, _ = O.init_detector(33, 1.2, (90.0, 30.0, 0.0),
                                       ("psi", "phi", "None"))
    psis = np.linspace(0.0, 180.0, 24, endpoint=False)
    images = {}
    for name, workers in (("serial", 0), ("threads", 4)):
        m = shared((33, 33))
        try:
            args = [(iq, qx, qy, qz, x0, y0, z0, ps, 1.0 / len(psis), 12.0,
                     1.0, 3.0, 1.0, m.name) for ps in psis]
            if workers:
                with ThreadPoolExecutor(max_workers=workers) as pool:
                    list(pool.map(D.generate_detector_ints, args))
            else:
                for a in args:
                    D.generate_detector_ints(a)
            images[name] = read(m, (33, 33))
        finally:
            free(m)
    assert rel_l2(images["threads"], images["serial"]) <= 1e-14


def test_concurrent_voxel_calls_on_per_thread_contexts():
    """Three threads call voxelgridmaker_fitting twice each on their own
    structure while the others run; the second call of each replays its
    recorded graph.  Every thread works on a context of its own, and every
    result equals a plan made for it alone."""
    rng = np.random.default_rng(23)
    structs = [W.graphite_slab(e, rng, disp_sigma=0.05)[0]
               for e in ((10.0, 12.0, 9.0), (13.0, 9.0, 11.0), (9.0, 9.0, 12.0))]
    kw = dict(r_voxel_size=0.5, q_voxel_size=0.15, max_q=1.5, energy=10000.0)
    phis = np.linspace(0.0, 180.0, 12, endpoint=False)

    def fresh(xyz):
        geom = F.VoxelGeometry(0.5, 0.15, 1.5)
        fv = F.element_f_values(["C"] * len(xyz), 10000.0)
        p = F.VoxelPlan(geom, [(xyz, fv, None)], phis=phis, smooth=1.0)
        try:
            p.set_atoms()
            p.execute()
            return p.iq().copy()
        finally:
            p.close()

    ref = [fresh(x) for x in structs]
    main_ctx = N.default_context()
    start = threading.Barrier(len(structs))
    seen = [None] * len(structs)

    def work(i):
        start.wait(timeout=60)
        seen[i] = id(N.default_context())
        res = []
        for _ in range(2):
            iq, _, _, _ = C.voxelgridmaker_fitting(structs[i], ["C"] * len(structs[i]),
                                                   smooth=1.0, phis=phis, **kw)
            res.append(iq.copy())
        return res

    size = C.PLAN_CACHE.size
    C.PLAN_CACHE.clear()
    C.PLAN_CACHE.size = 8               # each thread finds its own plan again
    try:
        with ThreadPoolExecutor(max_workers=len(structs)) as pool:
            results = list(pool.map(work, range(len(structs))))
        graphs = [p.graph_captured for p in C.PLAN_CACHE._plans.values()]
    finally:
        C.PLAN_CACHE.clear()
        C.PLAN_CACHE.size = size
    assert len(set(seen)) == len(structs) and id(main_ctx) not in seen
    assert graphs == [True] * len(structs)
    for i, res in enumerate(results):
        for iq in res:
            assert rel_l2(iq, ref[i]) <= 1e-9, i
