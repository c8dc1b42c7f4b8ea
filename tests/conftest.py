"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    """The C++ restatement of the reference path (built on demand)."""
    from oracle import spo
    spo.build("port")
    return spo.Oracle("port")


@pytest.fixture(scope="session")
def ref():
    """The compiled reference itself; only where the reference tree is present."""
    from oracle import spo
    if not os.path.isdir(spo.REF_TREE):
        pytest.skip("reference tree not present on this host")
    spo.build("ref")
    return spo.Oracle("ref")


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library; GPU tests fail (not skip) when it cannot be built or loaded."""
    from spica_gb300 import build, gpu
    build.build()
    return gpu.load_library()
