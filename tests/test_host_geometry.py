"""Host-side geometry of the product (giwaxsim_gb300.forward) against the
oracle and the reference-derived fixtures.  CPU only."""
import numpy as np
import pytest

from giwaxsim_gb300 import forward as F
from giwaxsim_gb300 import workloads as W
from giwaxsim_gb300.tools import comparison, utilities
from oracle import giwaxs_oracle as O
from tests.conftest import golden

GEOMS = [(0.3, 0.03, 3.0), (0.25, 0.02, 4.0), (0.3, 0.04095, 3.0),
         (0.2, 0.015, 2.5), (0.5, 0.15, 1.5), (0.3, 0.02, 2.0)]


@pytest.mark.parametrize("r,dq,mq", GEOMS)
def test_geometry_matches_oracle(r, dq, mq):
    g = F.VoxelGeometry(r, dq, mq)
    gs, q, phis = O.voxel_geometry(r, dq, mq)
    assert g.grid_size == gs
    assert np.array_equal(g.q, q)
    assert np.array_equal(g.auto_phis, phis)
    sub, qs, _, _ = O.downselect_voxelgrid(np.zeros((len(q),) * 3, np.int8),
                                           q, q, q, mq)
    assert np.array_equal(g.q_crop, qs)
    assert g.dq == np.diff(q)[0]


def test_geometry_errors():
    with pytest.raises(Exception, match="Max_q is non-physical"):
        F.VoxelGeometry(1.0, 0.1, 10.0)
    g = F.VoxelGeometry(0.5, 0.15, 1.5)
    with pytest.raises(Exception, match="real-space bounds smaller"):
        g.check_bounds(np.array([[0, 0, 0], [100.0, 100.0, 100.0]]))


def test_empty_atom_list_raises_before_device_work(monkeypatch):
    """An empty structure fails as the reference's bounds reduction fails
    (numpy max of an empty array, comparison.py:712-714), on the host,
    before any plan or device call."""
    from giwaxsim_gb300 import _native as N

    def no_device():
        raise AssertionError("device library reached")
    monkeypatch.setattr(N, "lib", no_device)
    with pytest.raises(ValueError, match="zero-size array"):
        comparison.voxelgridmaker_fitting(np.zeros((0, 3)), np.array([], "<U2"),
                                          0.3, 0.03, 3.0, 10000)


def test_phi_table_matches_reference_scalars():
    g = F.VoxelGeometry(0.3, 0.03, 3.0)
    phis = np.concatenate([g.auto_phis[:50], [0.0, 45.0, 90.0, 91.0, 135.0,
                                              179.5]])
    t = g.phi_table(phis)
    for i, phi in enumerate(phis):
        pr = np.radians(phi)
        assert t["cos_phi"][i] == np.cos(pr) and t["sin_phi"][i] == np.sin(pr)
        hx, hy, _ = O.slice_axes(g.grid_size, 0.3, phi)
        assert t["right_qy"][i] == hy[-1] and t["right_qx"][i] == hx[-1]
        p = phi - 90 if phi > 90 else phi
        tr, pa = np.deg2rad(90 - p), np.deg2rad(p)
        assert t["tan_t"][i] == np.tan(tr) and t["tan_p"][i] == np.tan(pa)
        assert t["cos_t"][i] == np.cos(tr) and t["sin_p"][i] == np.sin(pa)
        assert t["cl_swap"][i] == (phi > 90)


def test_phi_table_reuse():
    """A call with the phis and geometry of the last one gets the same
    (read-only) table; other phis or another geometry a fresh one, equal to
    a table made from scratch."""
    g = F.VoxelGeometry(0.3, 0.03, 3.0)
    phis = np.linspace(0.0, 179.0, 180)
    t1 = g.phi_table(phis)
    t2 = g.phi_table(phis.copy())
    assert t2 is t1 and not t1.flags.writeable
    assert t1.tobytes() == g._phi_table(phis).tobytes()
    t3 = g.phi_table(phis[:-1])
    assert t3 is not t1 and t3.tobytes() == g._phi_table(phis[:-1]).tobytes()
    g2 = F.VoxelGeometry(0.25, 0.02, 4.0)  # another h_max
    t4 = g2.phi_table(phis[:-1])
    assert t4 is not t3 and t4.tobytes() == g2._phi_table(phis[:-1]).tobytes()


def test_structure_constants_match_oracle():
    for name in ("graphite-50A", "si-100A"):
        xyz, el, _ = W.structures(name)[0]
        fv = F.element_f_values(el, 10000.0)
        xb, yb, zb, avg, mv = F.structure_constants(xyz, fv, 0.3)
        oxb, oyb, ozb, oavg = O.structure_constants(xyz, fv, 0.3)
        assert (xb, yb, zb, avg) == (oxb, oyb, ozb, oavg)
        assert mv == np.sqrt(xb ** 2 + yb ** 2) // 0.3


@pytest.mark.parametrize("elements", [
    np.array(["Si"] * 50),
    np.array(["C", "H", "O", "C", "N", "H", "C"] * 9),
    ["S", "O", "O", "Si", "C"] * 4,
    np.array(["C", "Si", "Cl"], dtype="<U3"),
    np.array(["Si", "Sn", "S", "Si", "Sn", "C", "S", "Sn"])[::2],  # strided
    np.array(["H"])])
def test_element_kinds_match_numpy_unique(elements):
    uniq, inv = F.element_kinds(elements)
    ref_u, ref_inv = np.unique(np.asarray(elements), return_inverse=True)
    assert np.array_equal(np.asarray(uniq)[inv], ref_u[ref_inv.reshape(-1)])
    assert sorted(uniq) == list(ref_u)
    if all(e in ("Si", "C", "H", "O", "N", "S") for e in uniq):
        fv = F.element_f_values(elements, 10000.0)
        z = {"Si": 14, "C": 6, "H": 1, "O": 8, "N": 7, "S": 16}
        assert np.array_equal(fv, np.array([z[str(e)] for e in np.asarray(elements)],
                                           dtype=complex))


def test_detector_corner_matrices_match_full_plane():
    """Rotation matrices from the tracked corners equal the ones the
    reference builds from the full rotated plane."""
    x, y, z, h, v = O.make_detector(2.0, 33, 2.0, 33)
    c = F.PlaneCorners(h, v)
    for kind, ang in [("psi", 90.0), ("phi", 30.0), ("theta", 10.0),
                      ("psi", 17.0), ("theta", 0.0), ("phi", 123.0)]:
        Rf = O.axis_matrix(x, y, z, kind, ang)
        Rc = c.matrix(kind, ang)
        assert np.array_equal(Rf, Rc), (kind, ang)
        x, y, z = O.fma_xyz(x, y, z, Rf)
        c = c.rotate(Rc)


def test_config_parsing(tmp_path):
    p = tmp_path / "cfg.txt"
    p.write_text("# comment\nr_voxel_size=0.3\nfill_bkg=True\nkey=a=b\n\n")
    cfg = utilities.parse_config_file(str(p))
    assert cfg == {"r_voxel_size": "0.3", "fill_bkg": "True", "key": "a=b"}
    assert utilities.str_to_bool("Yes") is True
    assert utilities.str_to_bool("off") is False
    assert utilities.str_to_bool("maybe") is False
    with pytest.raises(ValueError):
        utilities.str_to_bool("maybe", default=None)


def test_trim_and_rebin_weights_vs_reference():
    """trim_sim_data and the griddata weights (host parts of the
    comparison step) against the reference's own outputs, bit for bit."""
    from giwaxsim_gb300.tools.comparison import rebin_weights, trim_sim_data
    d = golden("golden_compare.npz")
    s, h, v = trim_sim_data(d["sim"], d["det_h"], d["det_v"], d["exp_qxy"], d["exp_qz"])
    assert np.array_equal(s, d["sim_trim"]) and np.array_equal(h, d["h_trim"])
    assert np.array_equal(v, d["v_trim"])
    idx, w = rebin_weights(h, v, d["exp_qxy"], d["exp_qz"])
    val = d["exp_img"].ravel()
    out = ((w[:, 0] * val[idx[:, 0]]) + w[:, 1] * val[idx[:, 1]]) + w[:, 2] * val[idx[:, 2]]
    out[idx[:, 0] < 0] = np.nan
    assert np.array_equal(out.reshape(s.shape), d["rebin_raw"], equal_nan=True)


def test_plan_inputs_equal_with_ranges_given():
    """The drop-in computes each structure's coordinate ranges once and hands
    them to the plan; the plan's structure table is the same either way."""
    xyz, el, wt = W.structures("graphite-50A")[0]
    g = F.VoxelGeometry(0.3, 0.03, 3.0)
    fv = F.element_f_values(el, 10000.0)

    class NoContext:
        handle = None
    kw = dict(phis=np.arange(7.0), fill_bkg=True, smooth=1.0, ctx=NoContext(),
              create=False)
    a = F.VoxelPlan(g, [(xyz, fv, wt)], **kw)
    b = F.VoxelPlan(g, [(xyz, fv, wt)], ranges=[F.coord_ranges(xyz)], **kw)
    assert a.structs.tobytes() == b.structs.tobytes()
    assert a.key()[1:] == b.key()[1:]


def test_plan_keeps_its_own_atoms():
    """A plan's coordinates and f values are its own copies (one structure
    or several): the caller changing its arrays afterwards changes neither
    what set_atoms() uploads nor the plan's key."""
    xyz, el, _ = W.structures("graphite-50A")[0]
    g = F.VoxelGeometry(0.3, 0.03, 3.0)

    class NoContext:
        handle = None
    kw = dict(phis=np.arange(5.0), ctx=NoContext(), create=False)
    for n_struct in (1, 2):
        coords = [np.array(xyz[:200 + 50 * i]) for i in range(n_struct)]
        fvs = [F.element_f_values(el[:200 + 50 * i], 10000.0) for i in range(n_struct)]
        plan = F.VoxelPlan(g, [(c, f, None) for c, f in zip(coords, fvs)], **kw)
        x0, f0, k0 = plan.xyz.copy(), plan.f.copy(), plan.key()
        for c, f in zip(coords, fvs):
            c += 1.0
            f *= 2.0
        assert np.array_equal(plan.xyz, x0) and np.array_equal(plan.f, f0)
        assert plan.key() == k0
        assert plan.xyz.flags.c_contiguous and plan.f.dtype == np.float32
        assert len(plan.f) == 2 * len(plan.xyz)


def test_missing_xraydb_refuses_without_opt_in(monkeypatch):
    """Without xraydb the f', f'' lookup (utilities.py:342-366) raises, as
    the reference's module-level `import xraydb` (utilities.py:3) does,
    unless the caller opts in to f' = f'' = 0 or passes a table."""
    if utilities._xraydb() is not None:
        pytest.skip("xraydb is installed")
    monkeypatch.setattr(utilities, "_ZERO_F1F2", [False])
    with pytest.raises(ImportError, match="xraydb"):
        utilities.get_element_f1_f2_dict(10000.0, ["C", "Si"])
    with pytest.raises(ImportError, match="xraydb"):
        F.element_f_values(["C", "Si"], 10000.0)
    f = F.element_f_values(["C", "Si", "C"], 10000.0,
                           {"C": 0.25 + 0.5j, "Si": -1.0 + 2.0j})
    assert np.array_equal(f, np.array([6.25 + 0.5j, 13.0 + 2.0j, 6.25 + 0.5j]))
    utilities.use_zero_f1f2()
    assert utilities.get_element_f1_f2_dict(10000.0, ["C"]) == {"C": 0j}
    utilities.use_zero_f1f2(False)
    with pytest.raises(ImportError, match="xraydb"):
        utilities.get_element_f1_f2_dict(10000.0, ["C"])
