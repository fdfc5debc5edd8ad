import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    lib = os.path.join(ROOT, "immerseflow_gb300", "libimmerseflow_gb300.so")
    orc = os.path.join(ROOT, "oracle", "liboracle.so")
    if not os.path.exists(orc):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    if not os.path.exists(lib):
        from immerseflow_gb300 import build

        build.build()


_ensure_built()


@pytest.fixture(scope="session")
def oracle():
    import _oracle

    return _oracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(TESTS, "golden", "results_52x52.npz"))


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(TESTS, "golden")
