"""Drop-in stage drivers with the reference's signatures
(tools/comparison.py of the reference):

  voxelgridmaker_fitting   comparison.py:673-788  -> GPU voxel plan
  detectormaker_fitting    comparison.py:790-870  -> GPU detector plan
  slabmaker_fitting        comparison.py:595-671  -> GPU slab (gw_slab)
  optimize_scale_offset    comparison.py:873-882  (host least squares)

Keyword-only extensions (all default to the reference's behaviour):
  phis=            explicit rotation list instead of the automatic count
  mode=            'batched' (default) or 'plain' (per-rotation, full grid)
  accum=           'fp64' (default) or 'kahan32' accumulation
  exact=           detector: replay the float64 index chain for every sample
                   instead of only the samples the float32 path cannot decide
  weights=         per-atom occupancy multiplying the scattering factor
  ctx=             a giwaxsim_gb300._native.Context
"""
import numpy as np

from ..forward import (PLAN_CACHE, DetectorPlan, Slab, VoxelGeometry, VoxelPlan,
                       coord_ranges, element_f_values)
from .utilities import calc_real_space_abc, load_pdb, load_xyz


def voxelgridmaker_fitting(coords, elements, r_voxel_size, q_voxel_size, max_q,
                           energy, num_cpus=None, fill_bkg=False, smooth=0, *,
                           phis=None, mode="batched", accum="fp64",
                           weights=None, f1f2=None, batch_slices=0, ctx=None):
    """I(q) on the cropped cube |q_i| < max_q + dq, C order (qy, qx, qz),
    with the carbon f0(q)^2 factor; returns (iq, qx, qy, qz) like the
    reference.  num_cpus is accepted and ignored (one GPU)."""
    geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
    coords = np.asarray(coords, dtype=np.float64)
    rg = coord_ranges(coords)
    geom.check_bounds(coords, rg)
    fv = element_f_values(elements, energy, f1f2)
    plan = PLAN_CACHE.checkout(geom, [(coords, fv, weights)], phis=phis,
                               fill_bkg=fill_bkg, smooth=smooth, mode=mode,
                               accum=accum, batch_slices=batch_slices, ctx=ctx,
                               ranges=[rg])
    ok = False
    try:
        plan.set_atoms()
        # a plan used a second time is recorded as one CUDA graph (its
        # launches depend on the plan only; the atoms are in its buffers)
        # and replayed from then on
        if plan.reused and not plan.graph_captured:
            plan.capture_graph()
        plan.execute()
        iq = plan.iq()
        ok = True
    finally:
        PLAN_CACHE.give_back(plan, ok)
    q = geom.q_crop
    return iq, q.copy(), q.copy(), q.copy()


def voxelgridmaker_average(structures, r_voxel_size, q_voxel_size, max_q,
                           energy, fill_bkg=False, smooth=0, *, phis=None,
                           accum="fp64", f1f2=None, batch_slices=0,
                           f0_element="C", ctx=None):
    """I(q) averaged over several structures before the f0 factor, as the
    legacy input_folder mode does (old_modules/voxelgridmaker.py:56-72).
    structures: list of (coords, elements) or (coords, elements, weights).
    All slices of all structures run in one batched plan."""
    geom = VoxelGeometry(r_voxel_size, q_voxel_size, max_q)
    items = []
    for s in structures:
        coords, elements = np.asarray(s[0], dtype=np.float64), s[1]
        w = s[2] if len(s) > 2 else None
        items.append((coords, element_f_values(elements, energy, f1f2), w))
    plan = VoxelPlan(geom, items, phis=phis, fill_bkg=fill_bkg, smooth=smooth,
                     accum=accum, average=True, f0_element=f0_element,
                     batch_slices=batch_slices, ctx=ctx)
    try:
        plan.set_atoms()
        plan.execute()
        iq = plan.iq()
    finally:
        plan.close()
    q = geom.q_crop
    return iq, q.copy(), q.copy(), q.copy()


def _weights(path, angles):
    return np.load(path) if path else np.ones_like(angles) / len(angles)


def detectormaker_fitting(iq, qx, qy, qz, num_pixels, max_q, angle_init_vals,
                          angle_init_axs, psis, psi_weights_path, phis,
                          phi_weights_path, thetas, theta_weights_path,
                          mirror=True, *, accum="fp64", exact=False,
                          ctx=None):
    """Detector image summed over psi x phi x theta orientations; returns
    (det_sum (num_pixels, num_pixels), det_h, det_v) like the reference."""
    psis, phis, thetas = (np.atleast_1d(np.asarray(a)) for a in (psis, phis, thetas))
    psi_w = _weights(psi_weights_path, psis)
    phi_w = _weights(phi_weights_path, phis)
    theta_w = _weights(theta_weights_path, thetas)
    assert len(psis) == len(psi_w), "psi weights length must equal psi_num"
    assert len(phis) == len(phi_w), "phi weights length must equal phi_num"
    assert len(thetas) == len(theta_w), "theta weights length must equal theta_num"
    assert np.abs(1 - np.sum(psi_w)) < 0.01, "psi weights must sum to 1"
    assert np.abs(1 - np.sum(phi_w)) < 0.01, "phi weights must sum to 1"
    assert np.abs(1 - np.sum(theta_w)) < 0.01, "theta weights must sum to 1"
    iq = np.asarray(iq)
    plan = DetectorPlan(iq.shape, qx, qy, qz, num_pixels, max_q,
                        angle_init_vals, angle_init_axs, psis, psi_w, phis,
                        phi_w, thetas, theta_w, mirror=mirror, accum=accum,
                        exact=exact, ctx=ctx)
    try:
        plan.set_iq(iq)
        plan.execute()
        det = plan.result()
    finally:
        plan.close()
    return det, plan.det_h.copy(), plan.det_v.copy()


def slabmaker_fitting(input_filepath, x_size, y_size, z_size, a, b, c, alpha,
                      beta, gamma, *, ctx=None):
    """Tile a unit cell into a slab of x/y/z size (comparison.py:595-671),
    on the device (gw_slab): same coordinates bit for bit, same atom order,
    same AssertionError messages."""
    if input_filepath.lower().endswith(".xyz"):
        coords, elements = load_xyz(input_filepath)
    elif input_filepath.lower().endswith(".pdb"):
        coords, elements = load_pdb(input_filepath)
    else:
        raise Exception("Files must be a .pdb or .xyz file")
    vecs = np.array(calc_real_space_abc(a, b, c, alpha, beta, gamma))
    slab = Slab(coords, vecs, (x_size, y_size, z_size), ctx=ctx)
    try:
        xyz, src = slab.coords()
    finally:
        slab.close()
    return xyz, np.asarray(elements)[src]


def trim_sim_data(sim_det_ints, det_h, det_v, exp_qxy, exp_qz):
    """Rows/columns of the simulated image inside the experiment's q range
    (comparison.py:161-191)."""
    h_mask, v_mask = _trim_masks(det_h, det_v, exp_qxy, exp_qz)
    return (np.asarray(sim_det_ints)[v_mask, :][:, h_mask], det_h[h_mask],
            det_v[v_mask])


def _trim_masks(det_h, det_v, exp_qxy, exp_qz):
    h_mask = (det_h >= np.min(exp_qxy)) & (det_h <= np.max(exp_qxy))
    v_mask = (det_v >= np.min(exp_qz)) & (det_v <= np.max(exp_qz))
    return h_mask, v_mask


def rebin_weights(qxy1, qz1, qxy2, qz2):
    """The linear interpolation griddata(points2, values, grid1) performs
    (comparison.py:425-438: a Delaunay triangulation of the experimental
    (qxy, qz) points and barycentric weights in the containing triangle),
    as 3 (index, weight) pairs per target pixel of the (qz1, qxy1) grid;
    index -1 outside the triangulation (griddata's NaN)."""
    from scipy.spatial import Delaunay
    g1x, g1z = np.meshgrid(qxy1, qz1)
    g2x, g2z = np.meshgrid(qxy2, qz2)
    points2 = np.vstack((g2x.ravel(), g2z.ravel())).T
    tri = Delaunay(points2)
    xi = np.stack([g1x.ravel(), g1z.ravel()], 1)
    s = tri.find_simplex(xi)
    T = tri.transform[s]
    d = xi - T[:, 2]
    c0 = T[:, 0, 0] * d[:, 0] + T[:, 0, 1] * d[:, 1]
    c1 = T[:, 1, 0] * d[:, 0] + T[:, 1, 1] * d[:, 1]
    w = np.stack([c0, c1, (1.0 - c0) - c1], 1)
    idx = tri.simplices[s].astype(np.int32)
    idx[s < 0] = -1
    w[s < 0] = 0.0
    return np.ascontiguousarray(idx), np.ascontiguousarray(w)


def _bilinear_map(shape_in, rows, cols):
    """map_coordinates(image, (rows, cols), order=1, cval=0) for every image
    of shape `shape_in` as (idx (n, 4) int32 flat input indices, -1 unused;
    w (n, 4)): the four neighbours (r0, c0), (r0, c0+1), (r0+1, c0),
    (r0+1, c0+1), r0 = floor(row).  The weights are scipy's own: an image
    that is 1 on the pixels of one (row, column) parity class and 0 elsewhere
    returns, at each point, the weight of its one neighbour in that class."""
    from scipy.ndimage import map_coordinates
    H, W = shape_in
    rows = np.asarray(rows, dtype=np.float64).ravel()
    cols = np.asarray(cols, dtype=np.float64).ravel()
    r0 = np.floor(rows).astype(np.int64)
    c0 = np.floor(cols).astype(np.int64)
    ii = np.arange(H)[:, None] % 2
    jj = np.arange(W)[None, :] % 2
    probe = {}
    for a in (0, 1):
        for b in (0, 1):
            img = ((ii == a) & (jj == b)).astype(np.float64)
            out = np.zeros(len(rows))
            map_coordinates(img, (rows, cols), order=1, output=out, cval=0)
            probe[a, b] = out
    idx = np.full((len(rows), 4), -1, dtype=np.int32)
    w = np.zeros((len(rows), 4))
    for k, (di, dj) in enumerate(((0, 0), (0, 1), (1, 0), (1, 1))):
        pr, pc = r0 + di, c0 + dj
        ok = (pr >= 0) & (pr < H) & (pc >= 0) & (pc < W)
        for a in (0, 1):
            for b in (0, 1):
                sel = ok & (pr % 2 == a) & (pc % 2 == b)
                w[sel, k] = probe[a, b][sel]
        use = ok & (w[:, k] != 0)
        idx[use, k] = (pr * W + pc)[use]
        w[~use, k] = 0.0
    return idx, w


def shift_peak_maps(det_h, det_v, shape, pad_width_qspace, pad_range_qspace):
    """The fixed parts of shift_peak (comparison.py:566-592) for a trimmed
    image of `shape` on the (det_v, det_h) grid: the polar warp of
    linear_polar (:469-499; centre at the pixel nearest q = 0, radius the
    image diagonal, output round(2 pi radius) x round(radius)), the column
    map of add_pad (:540-563) and the inverse warp of polar_linear
    (:501-538).  Returns dict(n_t, n_r, p_idx, p_w, col_src, q_idx, q_w)."""
    from scipy.ndimage import map_coordinates
    det_h, det_v = np.asarray(det_h), np.asarray(det_v)
    rows, cols = shape
    radius = float(np.sqrt(rows ** 2 + cols ** 2))
    ctr = np.array([int(np.argmin(np.abs(det_v))), int(np.argmin(np.abs(det_h)))])
    n_t, n_r = int(round(radius * 2 * np.pi)), int(round(radius))
    rr = np.linspace(0, radius, n_r)
    tt = np.linspace(0, 2 * np.pi, n_t)
    pc = rr * np.cos(tt[:, None]) + ctr[1]
    pr = rr * np.sin(tt[:, None]) + ctr[0]
    p_idx, p_w = _bilinear_map((rows, cols), pr, pc)
    # r axis: row 0 of the polar warp of |q|
    hh, vv = np.meshgrid(det_h, det_v)
    r_axis = np.zeros(n_r)
    map_coordinates(np.hypot(hh, vv), (pr[0], pc[0]), order=1, output=r_axis, cval=0)
    col_src = np.arange(n_r)
    steps = np.diff(r_axis)
    px = np.mean(steps[steps > 0])
    n_pad = int(np.round(pad_width_qspace / px))
    if n_pad:
        lo, hi = pad_range_qspace
        i0 = int(np.argmin(np.abs(r_axis - lo)))
        i1 = int(np.argmin(np.abs(r_axis - hi)))
        gap = int((i1 - i0 - 1) / n_pad - 1)
        assert gap >= 0, "pad_range is too small for desired pad_width"
        for k in range(n_pad):
            at = i0 + 2 * k + gap * k
            col_src = np.insert(col_src, at + 1, col_src[at])
        col_src = col_src[:-n_pad]
    yy, xx = np.mgrid[:rows, :cols] - ctr[:, None, None]
    rad = np.sqrt(yy ** 2 + xx ** 2)
    ang = np.arctan2(yy, xx)
    ang[ang < 0] += 2 * np.pi
    rad = (rad / n_r) * (n_r - 1)
    ang = (ang / (2 * np.pi)) * (n_t - 1)
    q_idx, q_w = _bilinear_map((n_t, n_r), ang, rad)
    return dict(n_t=n_t, n_r=n_r, p_idx=p_idx, p_w=p_w,
                col_src=np.ascontiguousarray(col_src, dtype=np.int32),
                q_idx=q_idx, q_w=q_w)


class Warp:
    """shift_peak of one trimmed-image geometry on the device (gw_warp)."""

    def __init__(self, det_h, det_v, shape, pad_width_qspace, pad_range_qspace,
                 ctx=None):
        import ctypes
        from .. import _native as N
        self._N = N
        self.ctx = ctx or N.default_context()
        self.shape = tuple(int(v) for v in shape)
        m = shift_peak_maps(det_h, det_v, self.shape, pad_width_qspace,
                            pad_range_qspace)
        h = ctypes.c_void_p()
        N.check(N.lib().gw_warp_create(
            self.ctx.handle, self.shape[0], self.shape[1], m["n_t"], m["n_r"],
            N.ptr(m["p_idx"]), N.ptr(m["p_w"]), N.ptr(m["col_src"]),
            N.ptr(m["q_idx"]), N.ptr(m["q_w"]), ctypes.byref(h)))
        self.handle = h

    def apply(self, image):
        N = self._N
        img = np.ascontiguousarray(image, dtype=np.float64)
        if img.shape != self.shape:
            raise ValueError("image shape differs from the warp's")
        out = np.empty_like(img)
        N.check(N.lib().gw_warp_apply(self.handle, N.ptr(img), 0, N.ptr(out), 0))
        return out

    def close(self):
        if getattr(self, "handle", None):
            self._N.lib().gw_warp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_WARPS = {}


def shift_peak(image, det_h, det_v, pad_width_qspace, pad_range_qspace, *,
               ctx=None):
    """Drop-in for comparison.py:566-592 on the device; the maps of a
    geometry are made once and kept."""
    det_h, det_v = np.asarray(det_h, np.float64), np.asarray(det_v, np.float64)
    key = (det_h.tobytes(), det_v.tobytes(), np.shape(image),
           float(pad_width_qspace), tuple(float(v) for v in pad_range_qspace),
           id(ctx))
    w = _WARPS.get(key)
    if w is None:
        if len(_WARPS) > 8:
            for old in _WARPS.values():
                old.close()
            _WARPS.clear()
        w = _WARPS[key] = Warp(det_h, det_v, np.shape(image), pad_width_qspace,
                               pad_range_qspace, ctx=ctx)
    return w.apply(image)


class Comparison:
    """Device plan of the experimental comparison: the experiment rebinned
    once onto the trimmed simulation grid, then per simulated image the
    scale + offset least squares and residuals over the unmasked pixels
    (comparison.py:161-191, :406-445, :873-882; fit_slabsize.py:43-44)."""

    def __init__(self, det_h, det_v, exp_img, exp_qxy, exp_qz, exp_mask,
                 weights=None, shift=None, ctx=None):
        """shift: (pad_width, pad_range) to apply shift_peak to the trimmed
        simulated image first, as fit_slabsize.py:36 does; None: no warp."""
        import ctypes
        from .. import _native as N
        self._N = N
        self.ctx = ctx or N.default_context()
        det_h, det_v = np.asarray(det_h), np.asarray(det_v)
        h_mask, v_mask = _trim_masks(det_h, det_v, exp_qxy, exp_qz)
        hi, vi = np.where(h_mask)[0], np.where(v_mask)[0]
        if len(hi) == 0 or len(vi) == 0:
            raise ValueError("the simulated image does not overlap the experiment")
        self.h0, self.v0 = int(hi[0]), int(vi[0])
        self.rows, self.cols = len(vi), len(hi)
        self.n_v, self.n_h = len(det_v), len(det_h)
        self.det_h_trim, self.det_v_trim = det_h[hi], det_v[vi]
        if weights is None:
            weights = rebin_weights(self.det_h_trim, self.det_v_trim, exp_qxy, exp_qz)
        idx, w = weights
        vals = np.ascontiguousarray(np.asarray(exp_img, dtype=np.float64).ravel())
        mvals = np.ascontiguousarray(np.asarray(exp_mask, dtype=np.float64).ravel())
        h = ctypes.c_void_p()
        N.check(N.lib().gw_compare_create(
            self.ctx.handle, self.n_v, self.n_h, self.v0, self.h0, self.rows,
            self.cols, N.ptr(idx), N.ptr(w), N.ptr(vals), N.ptr(mvals),
            len(vals), ctypes.byref(h)))
        self.handle = h
        self.warp = None
        if shift is not None:
            self.warp = Warp(self.det_h_trim, self.det_v_trim,
                             (self.rows, self.cols), shift[0], shift[1],
                             ctx=self.ctx)
            N.check(N.lib().gw_compare_set_warp(self.handle, self.warp.handle))

    def target(self):
        """(rebinned map, rebinned mask) on the trimmed grid."""
        t = np.empty((self.rows, self.cols))
        m = np.empty((self.rows, self.cols), dtype=np.uint8)
        self._N.check(self._N.lib().gw_compare_target(self.handle, self._N.ptr(t),
                                                      self._N.ptr(m)))
        return t, m.astype(int)

    def evaluate(self, sim, on_device=False, residual=False):
        """(scale, offset, misfit, pixels used[, residual map]) for a whole
        simulated image (host (n_v, n_h) array or a device pointer)."""
        import ctypes
        N = self._N
        out = np.zeros(4)
        res = np.empty((self.rows, self.cols)) if residual else None
        if on_device:
            src = ctypes.c_void_p(sim)
        else:
            sim = np.ascontiguousarray(sim, dtype=np.float64)
            if sim.shape != (self.n_v, self.n_h):
                raise ValueError("sim must be the whole (n_v, n_h) image")
            src = N.ptr(sim)
        N.check(N.lib().gw_compare_eval(self.handle, src, int(bool(on_device)),
                                        N.ptr(out), N.ptr(res)))
        r = (float(out[0]), float(out[1]), float(out[2]), int(out[3]))
        return r + (res,) if residual else r

    def close(self):
        if getattr(self, "handle", None):
            self._N.lib().gw_compare_destroy(self.handle)
            self.handle = None
        if getattr(self, "warp", None) is not None:
            self.warp.close()
            self.warp = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _identity(shape):
    n = int(np.prod(shape))
    idx = np.repeat(np.arange(n, dtype=np.int32), 3).reshape(n, 3)
    w = np.zeros((n, 3))
    w[:, 0] = 1.0
    return idx, w


def rebin_qmap_and_mask(qxy1, qz1, qmap2, qxy2, qz2, qmap2_mask, *, ctx=None):
    """qmap2 and its mask rebinned onto the (qz1, qxy1) grid by linear
    interpolation (comparison.py:406-445); the weights are made on the host
    (Delaunay), the interpolation runs on the device."""
    c = _whole_grid(np.asarray(qxy1), np.asarray(qz1), qmap2, qxy2, qz2,
                    qmap2_mask, ctx)
    try:
        return c.target()
    finally:
        c.close()


def _whole_grid(qxy1, qz1, qmap2, qxy2, qz2, qmap2_mask, ctx):
    """A Comparison whose window is the whole (qz1, qxy1) grid."""
    c = Comparison.__new__(Comparison)
    import ctypes
    from .. import _native as N
    c._N = N
    c.ctx = ctx or N.default_context()
    c.v0 = c.h0 = 0
    c.rows, c.cols = len(qz1), len(qxy1)
    c.n_v, c.n_h = c.rows, c.cols
    idx, w = rebin_weights(qxy1, qz1, qxy2, qz2)
    vals = np.ascontiguousarray(np.asarray(qmap2, dtype=np.float64).ravel())
    mvals = np.ascontiguousarray(np.asarray(qmap2_mask, dtype=np.float64).ravel())
    h = ctypes.c_void_p()
    N.check(N.lib().gw_compare_create(c.ctx.handle, c.n_v, c.n_h, 0, 0, c.rows,
                                      c.cols, N.ptr(idx), N.ptr(w), N.ptr(vals),
                                      N.ptr(mvals), len(vals), ctypes.byref(h)))
    c.handle = h
    return c


def optimize_scale_offset(sim_map, rebin_map, rebin_mask, *, ctx=None):
    """Least-squares scale and offset of sim onto rebin where mask == 0
    (comparison.py:873-882), as a device reduction."""
    import ctypes
    from .. import _native as N
    sim = np.ascontiguousarray(sim_map, dtype=np.float64)
    ctx = ctx or N.default_context()
    idx, w = _identity(sim.shape)
    vals = np.ascontiguousarray(np.asarray(rebin_map, dtype=np.float64).ravel())
    mvals = np.ascontiguousarray((np.asarray(rebin_mask) != 0).astype(np.float64).ravel())
    h = ctypes.c_void_p()
    rows, cols = sim.shape
    N.check(N.lib().gw_compare_create(ctx.handle, rows, cols, 0, 0, rows, cols,
                                      N.ptr(idx), N.ptr(w), N.ptr(vals),
                                      N.ptr(mvals), len(vals), ctypes.byref(h)))
    out = np.zeros(4)
    try:
        N.check(N.lib().gw_compare_eval(h, N.ptr(sim), 0, N.ptr(out), None))
    finally:
        N.lib().gw_compare_destroy(h)
    return out[0], out[1]
