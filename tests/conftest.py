import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    # the synthetic structures and fixtures use f = Z (xraydb is not
    # installed here, and the fixtures were made with f' = f'' = 0)
    from giwaxsim_gb300.tools import utilities
    utilities.use_zero_f1f2()
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device (GB300, sm_103a) and the built "
        "native library")


def golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name))
