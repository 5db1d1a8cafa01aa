"""Shared fixtures.  `-m gpu` tests need a CUDA GPU; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native():
    import resmcm_ari_gb300 as rg
    rg.build()
    return rg


@pytest.fixture(scope="session")
def engine(native):
    eng = native.Engine(device=0)
    yield eng
    eng.close()
