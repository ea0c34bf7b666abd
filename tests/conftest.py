import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def sampler():
    if not gpu_available():
        pytest.skip("no GPU")
    from spin_dynamics_gb300.dynamics import TraceSampler
    s = TraceSampler(0)
    yield s
    s.close()


def iso_csr(oracle, sysp, Bz):
    e1, e2 = sysp.e1, sysp.e2
    return oracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, Bz, sysp.J, sysp.D, sysp.kS,
                              sysp.kT)


def general_csr(oracle, sysp, Bvec):
    e1, e2 = sysp.e1, sysp.e2
    return oracle.build_h_general(e1.g_I, e1.A, e1.gammas, e2.g_I, e2.A, e2.gammas, Bvec, sysp.J,
                                  sysp.D, sysp.kS, sysp.kT)
