"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the in-tree
libsgw_gb300.so; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libsgw_gb300.so")


@pytest.fixture(scope="session")
def lin_prob():
    """The reference's solver fixture (algo/linear_solver/test/lin_prob.xml.bz2)."""
    d = np.load(os.path.join(GOLDEN, "lin_prob.npz"))
    return d["A"], d["b"], d["sigma"]


@pytest.fixture(scope="session")
def c0_system():
    from sternheimergw_gb300 import synth
    return synth.config("c0")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, loaded without any fallback."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    from sternheimergw_gb300 import _capi
    return _capi.lib(build_if_missing=False)
