"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(os.path.join(ROOT, "tests", "golden", "golden.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import OracleLib
    return OracleLib("port")


@pytest.fixture(scope="session")
def tg():
    """The CUDA library, built in-tree if needed; fails loudly without it."""
    from topopt_gb300.build import build
    build()
    import topopt_gb300
    topopt_gb300.lib()
    return topopt_gb300
