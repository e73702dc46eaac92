"""Drop-in for the reference's tools/detector.py, on the GB300 library.

  make_detector              detector.py:5-29    (array construction)
  rotate_about_normal        detector.py:33-78   } axis from the plane's
  rotate_about_horizontal    detector.py:80-120  } corners, points rotated in
  rotate_about_vertical      detector.py:122-162 } the BLAS fused order
  intersect_detector         detector.py:194-232 -> gw_gather
  rotate_psi_phi_theta       detector.py:234-244
  mirror_vertical_horizontal detector.py:246-275 -> gw_mirror
  generate_detector_ints     detector.py:278-300 -> gw_gather (rotations +
                             weight) accumulated into the named image

The orientation-summed fast path is detectormaker_fitting in
tools/comparison.py.
"""
import threading
from multiprocessing import shared_memory

import numpy as np

from .. import _native as N
from ..forward import PlaneCorners


def make_detector(h_max, num_pixels_h, v_max, num_pixels_v):
    h = np.linspace(-h_max, h_max, num_pixels_h)
    v = np.linspace(-v_max, v_max, num_pixels_v)
    y, z = np.meshgrid(h, v)
    return np.zeros_like(y), y, z, h, v


def _rotate(det_x, det_y, det_z, kind, angle):
    c = PlaneCorners.from_grids(det_x, det_y, det_z)
    R = c.matrix(kind, angle)
    pts = np.stack([np.ravel(det_x), np.ravel(det_y), np.ravel(det_z)], 1)
    out = N.rotate_points(R, pts)
    shape = np.shape(det_x)
    return (out[:, 0].reshape(shape), out[:, 1].reshape(shape),
            out[:, 2].reshape(shape))


def rotate_about_normal(det_x_grid, det_y_grid, det_z_grid, psi):
    return _rotate(det_x_grid, det_y_grid, det_z_grid, "psi", psi)


def rotate_about_horizontal(det_x_grid, det_y_grid, det_z_grid, theta):
    return _rotate(det_x_grid, det_y_grid, det_z_grid, "theta", theta)


def rotate_about_vertical(det_x_grid, det_y_grid, det_z_grid, phi):
    return _rotate(det_x_grid, det_y_grid, det_z_grid, "phi", phi)


def rotate_psi_phi_theta(det_x, det_y, det_z, psi, phi, theta):
    x, y, z = rotate_about_normal(det_x, det_y, det_z, psi)
    x, y, z = rotate_about_vertical(x, y, z, phi)
    return rotate_about_horizontal(x, y, z, theta)


# held while an orientation's image is added into the named image
_IMAGE_ADD_LOCK = threading.Lock()


def _gather(iq, qx, qy, qz, x, y, z, mats=(), weight=None, ctx=None):
    ctx = ctx or N.default_context()
    iq = np.ascontiguousarray(iq, dtype=np.float64)
    shape = np.array(iq.shape, dtype=np.int32)
    qmin = np.array([np.min(qx), np.min(qy), np.min(qz)], dtype=np.float64)
    xs, ys, zs = (np.ascontiguousarray(np.ravel(a), dtype=np.float64)
                  for a in (x, y, z))
    R = np.ascontiguousarray(np.array(mats).reshape(-1, 9)) if len(mats) else None
    out = np.empty(len(xs))
    N.check(N.lib().gw_gather(ctx.handle, N.ptr(iq), N.ptr(shape), N.ptr(qmin),
                              float(np.diff(qz)[0]), N.ptr(xs), N.ptr(ys),
                              N.ptr(zs), len(xs), N.ptr(R), len(mats),
                              float(weight) if weight is not None else 1.0,
                              int(weight is not None), N.ptr(out)))
    return out.reshape(np.shape(x))


def intersect_detector(int_voxels, qx, qy, qz, det_x_grid, det_y_grid,
                       det_z_grid, ctx=None):
    """Nearest voxel of every detector pixel, clipped to the grid."""
    return _gather(int_voxels, qx, qy, qz, det_x_grid, det_y_grid, det_z_grid,
                   ctx=ctx)


def mirror_vertical_horizontal(qmap, ctx=None):
    """Four-fold fold of an image about its centre row and column."""
    ctx = ctx or N.default_context()
    q = np.ascontiguousarray(qmap, dtype=np.float64)
    out = np.empty_like(q)
    N.check(N.lib().gw_mirror(ctx.handle, N.ptr(q), q.shape[0], q.shape[1],
                              N.ptr(out)))
    return out


def generate_detector_ints(args, ctx=None):
    """One orientation's weighted image added into the named shared-memory
    image (detector.py:278-300).  args is the reference's 14-tuple."""
    (iq, qx, qy, qz, det_x, det_y, det_z, psi, psi_weight, phi, phi_weight,
     theta, theta_weight, det_ints_shm_name) = args
    c = PlaneCorners.from_grids(det_x, det_y, det_z)
    mats = []
    for kind, ang in (("psi", psi), ("phi", phi), ("theta", theta)):
        R = c.matrix(kind, ang)
        c = c.rotate(R)
        mats.append(R)
    det_int = _gather(iq, qx, qy, qz, det_x, det_y, det_z, mats,
                      psi_weight * phi_weight * theta_weight, ctx=ctx)
    shm = shared_memory.SharedMemory(name=det_ints_shm_name)
    try:
        det_ints = np.ndarray(np.shape(det_int), dtype=np.float64,
                              buffer=shm.buf)
        # the reference's thread pool adds orientations concurrently and
        # loses updates; here the additions are serialised
        with _IMAGE_ADD_LOCK:
            det_ints += det_int
        del det_ints
    finally:
        shm.close()
