"""End-to-end regression on the reference's shipped example: the PM6 slab
config (config_templates/simulate_GIWAXS_config.txt) through the drop-in
config driver, against the reference's own result on the same inputs
(f' = f'' = 0) and, loosely, against its shipped output (made with xraydb's
f', f'' at 12.7 keV, which this environment does not have)."""
import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu


def write_pdb(path, xyz, el, cell):
    with open(path, "w") as fh:
        fh.write("CRYST1%9.3f%9.3f%9.3f%7.2f%7.2f%7.2f\n" % tuple(cell))
        for i, ((x, y, z), e) in enumerate(zip(xyz, el)):
            line = "ATOM  %5d  %-3s RES A   1    %8.3f%8.3f%8.3f  1.00  0.00" % (
                i % 100000, e, x, y, z)
            fh.write(line.ljust(76) + "%2s\n" % e)


def test_pm6_example(tmp_path):
    from giwaxsim_gb300 import simulate_GIWAXS as S
    d = golden("golden_pm6.npz")
    pdb = tmp_path / "PM6_sample.pdb"
    write_pdb(pdb, d["cell_xyz"], d["cell_el"], d["cell"])
    cfg = dict(line.split("=", 1) for line in d["config"])
    cfg["input_filepath"] = str(pdb)
    cfg["save_folder"] = str(tmp_path / "out")
    # the slab the drop-in slabmaker builds is the reference's
    xs, ys, zs = (float(cfg[k]) for k in ("x_size", "y_size", "z_size"))
    slab, _ = S.slabmaker_fitting(str(pdb), xs, ys, zs, *d["cell"])
    assert len(slab) == int(d["slab_n"])
    assert np.array_equal(slab[:16], d["slab_head"])
    assert np.allclose(slab.sum(0), d["slab_sum"], rtol=1e-13)
    det, h, v = S.main(cfg)["PM6_sample"]
    assert np.array_equal(h, d["det_h"]) and np.array_equal(v, d["det_v"])
    ref = d["det_ref"]
    assert np.linalg.norm(det - ref) / np.linalg.norm(ref) <= 1e-5
    rel = np.abs(det - d["det_shipped"]) / np.abs(d["det_shipped"])
    assert np.median(rel) < 0.01 and np.percentile(rel, 99) < 0.05
