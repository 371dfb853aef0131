import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "montecarloradiativetransfer.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def M():
    import mcrt_gb300

    mcrt_gb300.lib()  # fails loudly when the library was not built
    return mcrt_gb300


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx(M):
    if M.lib().mcrt_device_count() <= 0:
        pytest.fail("the gpu tests need a CUDA device")
    return M.default_context()


@pytest.fixture(scope="session")
def mie5(M):
    """Mie spheres x = 5, m = 1.5 + 0.001i, 1801-angle tables."""
    return M.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)


@pytest.fixture(scope="session")
def mie2(M):
    """Mie spheres x = 2, m = 1.31, 1801-angle tables."""
    return M.MieScatterer(2.0 / (2 * math.pi), 1.31 + 0.0j, 1.0, 0.1, Ntheta=1801)
