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


def oracle_made_mie(M, O, x, m):
    """A library scatterer whose tables come from the oracle's own bhmie and calculate_csrn
    (as the Julia binding hands the library the tables that the reference's MieScatterer
    made), so that parity runs feed both sides one producer's tables and the library's
    producer is checked on its own against the oracle's."""
    o = O.MieScatterer(x / (2 * math.pi), m, 1.0, 0.1, Ntheta=1801)
    s = M.MieScatterer.from_tables(o.omega, o.kl, o.F11, o.F12, o.F33, o.F34, o.S11, o.S22, o.csrn)
    s.r, s.m, s.lam, s.nu, s.x, s.q_ext = o.r, o.m, o.lam, o.nu, o.x, o.q_ext
    return s


@pytest.fixture(scope="session")
def mie5(M, O):
    """Mie spheres x = 5, m = 1.5 + 0.001i, 1801-angle tables (made by the oracle)."""
    return oracle_made_mie(M, O, 5.0, 1.5 + 0.001j)


@pytest.fixture(scope="session")
def mie2(M, O):
    """Mie spheres x = 2, m = 1.31, 1801-angle tables (made by the oracle)."""
    return oracle_made_mie(M, O, 2.0, 1.31 + 0.0j)
