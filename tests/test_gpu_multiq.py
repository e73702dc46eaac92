"""Multi-q atomic form factors (generate_voxel_grid_low_mem with
aff_num_qs > 1) on the device against the reference's own output
(tests/golden/golden_multiq.npz) and the oracle's per-shell restatement."""
import os

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300.tools import voxelgrids as V
from oracle import giwaxs_oracle as O
from tests.conftest import golden

pytestmark = pytest.mark.gpu

F1F2 = {"C": 0j, "O": 0j}
TOL = 1e-5  # normwise, float32 transforms against float64


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _xyz_file(tmp_path, d):
    path = os.path.join(tmp_path, "mq.xyz")
    with open(path, "w") as fh:
        fh.write("%d\nslab\n" % len(d["coords"]))
        for e, (x, y, z) in zip(d["elements"], d["coords"]):
            fh.write("%s %.17g %.17g %.17g\n" % (e, x, y, z))
    return path


@pytest.mark.parametrize("name", ["plain", "fillsmooth"])
def test_reference_mode_vs_reference_output(tmp_path, name):
    d = golden("golden_multiq.npz")
    iq, qx, qy, qz = V.generate_voxel_grid_low_mem(
        _xyz_file(str(tmp_path), d), float(d["r"]), float(d["dq"]),
        float(d["max_q"]), int(d[name + "_K"]), 10000.0, "mq",
        fill_bkg=bool(d[name + "_fill"]), smooth=int(d[name + "_smooth"]),
        f1f2=F1F2)
    ref = d[name + "_iq"]
    assert np.array_equal(qx, d["q"])
    assert iq.shape == ref.shape
    assert rel_l2(iq, ref) <= TOL
    # the doubled last shell: exactly where the reference doubles
    assert np.array_equal(iq == 0, ref == 0)


@pytest.mark.parametrize("name", ["plain", "fillsmooth"])
def test_per_shell_mode_vs_oracle(tmp_path, name):
    d = golden("golden_multiq.npz")
    K = int(d[name + "_K"])
    fill, smooth = bool(d[name + "_fill"]), int(d[name + "_smooth"])
    iq, q, _, _ = V.generate_voxel_grid_low_mem(
        _xyz_file(str(tmp_path), d), float(d["r"]), float(d["dq"]),
        float(d["max_q"]), K, 10000.0, "mq", fill_bkg=fill, smooth=smooth,
        f1f2=F1F2, aff_mode="per_shell")
    ref = O.voxelgrid_multi_q(d["coords"], d["elements"], F1F2, float(d["r"]),
                              float(d["dq"]), float(d["max_q"]), K,
                              fill_bkg=fill, smooth=smooth, mode="per_shell")
    assert rel_l2(iq, ref["iq"]) <= TOL
    outside = ~np.any(ref["masks"], axis=0)
    assert np.all(iq[outside] == 0.0)
    for k, m in enumerate(ref["masks"]):  # shell by shell
        assert rel_l2(iq[m], ref["shell_iq"][k][m]) <= TOL


def test_shell_state_errors():
    d = golden("golden_multiq.npz")
    geom = F.VoxelGeometry(float(d["r"]), float(d["dq"]), float(d["max_q"]))
    full = F.VoxelGeometry.from_axes(geom.grid_size, geom.r_voxel_size, geom.q)
    xyz = d["coords"]
    fv = np.full(len(xyz), 6.0 + 0j)
    plan = F.VoxelPlan(full, [(xyz, fv, None)], phis=[0.0, 30.0], f0_element=None,
                       real=False)  # shells need the general path
    lower, upper, fk = V.aff_shell_tables(geom.q, 3, d["elements"], 1e4, F1F2)
    avg = np.ones((3, 1), dtype=complex)
    with pytest.raises(N.GwError) as e:  # before set_atoms
        plan.set_shells(geom.q, lower, upper, fk, avg)
    assert e.value.status == N.GW_ERR_STATE
    plan.set_atoms()
    with pytest.raises(N.GwError) as e:  # decreasing shells
        plan.set_shells(geom.q, lower[::-1], upper[::-1], fk, avg)
    assert e.value.status == N.GW_ERR_ARG
    plan.set_shells(geom.q, lower, upper, fk, avg)
    plan.execute()
    a = plan.iq()
    plan.set_shells(None, None, None, None, None)  # cleared: f is stale
    with pytest.raises(N.GwError) as e:
        plan.execute()
    assert e.value.status == N.GW_ERR_STATE
    plan.set_atoms()
    plan.execute()
    b = plan.iq()
    assert not np.array_equal(a, b)
    plan.close()
