"""Slab construction on the device (gw_slab) against the reference's own
slabmaker_fitting (tests/golden/golden_slab.npz): every coordinate bit for
bit (SHA-256 of the float64 array), the atom order and the elements."""
import hashlib
import os

import numpy as np
import pytest

from giwaxsim_gb300 import _native as N
from giwaxsim_gb300 import forward as F
from giwaxsim_gb300.tools import comparison
from giwaxsim_gb300.tools.utilities import calc_real_space_abc
from tests.conftest import golden

pytestmark = pytest.mark.gpu
CASES = ["pm6", "graphite", "graphite_odd", "triclinic"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_device_slab_bit_exact(name):
    d = golden("golden_slab.npz")
    vecs = np.array(calc_real_space_abc(*d[name + "_cellp"]))
    slab = F.Slab(d[name + "_cell_xyz"], vecs, d[name + "_size"])
    xyz, src = slab.coords()
    assert slab.n == int(d[name + "_n"])
    assert np.array_equal(xyz[:8], d[name + "_head"])
    assert sha(xyz) == str(d[name + "_sha"])
    els = np.asarray(d[name + "_cell_el"])[src]
    assert hashlib.sha256("".join(els.tolist()).encode()).hexdigest() == str(d[name + "_el_sha"])
    ext = xyz.max(0) - xyz.min(0)
    assert np.array_equal(slab.bounds, ext)
    slab.close()


def test_dropin_slabmaker_from_file(tmp_path):
    d = golden("golden_slab.npz")
    name = "triclinic"
    path = os.path.join(tmp_path, "cell.xyz")
    with open(path, "w") as fh:
        cx, ce = d[name + "_cell_xyz"], d[name + "_cell_el"]
        fh.write("%d\ncell\n" % len(cx))
        for e, (x, y, z) in zip(ce, cx):
            fh.write("%s %.17g %.17g %.17g\n" % (e, x, y, z))
    xyz, els = comparison.slabmaker_fitting(path, *d[name + "_size"],
                                            *d[name + "_cellp"])
    assert sha(xyz) == str(d[name + "_sha"])
    assert len(els) == len(xyz)


def test_slab_argument_errors():
    with pytest.raises(N.GwError):
        F.Slab(np.zeros((1, 3)), np.eye(3) * -1.0, (10.0, 10.0, 10.0))
