"""The evaluation order of the reference's BLAS rotations on this host.

The reference rotates point sets with BLAS products: np.dot(coords, R.T)
for the atoms (tools/utilities.py:315) and R @ np.vstack([x, y, z]) for the
detector (tools/detector.py:71,113,155).  Voxel and detector indices come
from floor divisions of those products, so an index is bit-exact only if the
product is.  The oracle (oracle/oracle_fma.c) and the device (rot_chain,
rot_y) evaluate every output element as the fused chain
fma(p2, R[i][2], fma(p1, R[i][1], p0 * R[i][0])), the order OpenBLAS takes on
x86_64, where tests/golden/golden_rotation.npz was made by running the
reference.

These tests compare this host's numpy with that chain bit for bit, on the
fixture's inputs and on 10^5 random points per product, so that the parity
claim is recorded for every host the tests run on.  The copy marked gpu runs
on the GPU machine's host (aarch64), where the GPU tests run.
"""
import platform

import numpy as np
import pytest

from oracle import giwaxs_oracle as O
from tests.conftest import golden


def _host():
    return "%s, numpy %s" % (platform.machine(), np.__version__)


def _random_cases(seed=7, n=100_000):
    rng = np.random.default_rng(seed)
    for _ in range(4):
        pts = rng.uniform(-200.0, 200.0, (n, 3))
        pts[: n // 4] *= 1e-3          # small magnitudes as well
        pr = np.radians(rng.uniform(0, 180))
        Rz = np.array([[np.cos(pr), -np.sin(pr), 0],
                       [np.sin(pr), np.cos(pr), 0], [0, 0, 1]])
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        Ru = O.rotation_matrix(u, np.radians(rng.uniform(-180, 180)))
        yield pts, Rz
        yield pts, Ru


def _check_rows(pts, R):
    """np.dot(coords, R.T), utilities.py:315."""
    got = np.dot(pts, R.T)
    want = O.fma_rows(pts, R)
    bad = np.count_nonzero(got != want)
    assert bad == 0, ("np.dot(coords, R.T) differs from the fused chain in "
                      "%d of %d values on %s" % (bad, got.size, _host()))


def _check_xyz(x, y, z, R):
    """R @ np.vstack([x, y, z]), detector.py:71,113,155."""
    got = R @ np.vstack([x.ravel(), y.ravel(), z.ravel()])
    want = np.vstack([a.ravel() for a in O.fma_xyz(x, y, z, R)])
    bad = np.count_nonzero(got != want)
    assert bad == 0, ("R @ vstack(...) differs from the fused chain in %d of "
                      "%d values on %s" % (bad, got.size, _host()))


def _run_all():
    g = golden("golden_rotation.npz")
    coords = g["coords"]
    for phi in g["phis"]:
        pr = np.radians(phi)
        Rz = np.array([[np.cos(pr), -np.sin(pr), 0],
                       [np.sin(pr), np.cos(pr), 0], [0, 0, 1]])
        _check_rows(coords, Rz)
    for pts, R in _random_cases():
        _check_rows(pts, R)
        _check_xyz(pts[:, 0], pts[:, 1], pts[:, 2], R)


def test_blas_rotation_order_this_host():
    _run_all()


@pytest.mark.gpu
def test_blas_rotation_order_gpu_host():
    """The same check, collected with the GPU tests so that it runs on the
    host of the GPU machine."""
    _run_all()
