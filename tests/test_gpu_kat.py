"""Known-answer tests of the voxel stage that need no oracle: a single atom
scatters |f|^2 into every covered voxel, and two atoms stacked along z by n
voxels give |F|^2 = 2|f|^2 (1 + cos(2 pi k n / g)) for the slice row of
frequency k, averaged over the rows each qz voxel bins (process_file2's
floor((q - q_min) / dq) on the fftshift(fftfreq) axis)."""
import numpy as np
import pytest
from numpy.fft import fftfreq, fftshift

from giwaxsim_gb300 import forward as F

pytestmark = pytest.mark.gpu

PHIS = np.linspace(0.0, 180.0, 12, endpoint=False)


def _plan(geom, xyz, f):
    plan = F.VoxelPlan(geom, [(np.asarray(xyz, float), np.full(len(xyz), f), None)],
                       phis=PHIS, f0_element=None)
    plan.set_atoms()
    plan.execute()
    return plan


def test_single_atom_flat_intensity():
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    f = 6.0 + 2.0j
    with np.errstate(divide="ignore", invalid="ignore"):
        plan = _plan(geom, [[1.3, -0.4, 2.2]], f)
    iq, cnt = plan.iq(), plan.counts()
    plan.close()
    assert np.all(iq[cnt == 0] == 0.0)
    assert np.max(np.abs(iq[cnt > 0] / abs(f) ** 2 - 1.0)) < 1e-6
    assert (cnt > 0).mean() > 0.3  # 12 rotations cover about half the crop


@pytest.mark.parametrize("n", [1, 3, 7])
def test_two_atoms_z_fringes(n):
    geom = F.VoxelGeometry(0.5, 0.15, 1.5)
    r, g, q = geom.r_voxel_size, geom.grid_size, geom.q
    f = 5.0 + 0j
    with np.errstate(divide="ignore", invalid="ignore"):
        plan = _plan(geom, [[0.7, 0.2, 0.0], [0.7, 0.2, n * r]], f)
    iq, cnt = plan.iq(), plan.counts()
    plan.close()
    # rows of a slice: frequency index k (fftshift order) at q_v
    qv = fftshift(fftfreq(g, d=r) * 2 * np.pi)
    k = np.arange(g) - g // 2
    I_row = 2 * abs(f) ** 2 * (1 + np.cos(2 * np.pi * k * n / g))
    keep = (qv >= q.min()) & (qv <= q.max())
    dq = np.diff(q)[0]
    iz = ((qv[keep] - q.min()) // dq).astype(int)
    s = np.bincount(iz, weights=I_row[keep], minlength=len(q))
    c = np.bincount(iz, minlength=len(q))
    E = np.divide(s, c, out=np.zeros_like(s), where=c > 0)
    Ez = E[geom.crop_lo:geom.crop_hi + 1]
    exp = np.broadcast_to(Ez, iq.shape) * (cnt > 0)
    ok = cnt > 0
    assert np.all(iq[~ok] == 0.0)
    assert np.max(np.abs(iq[ok] - exp[ok])) <= 1e-5 * 4 * abs(f) ** 2
