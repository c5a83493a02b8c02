import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the CUDA library")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="session")
def lib():
    import milc_qcd_gb300 as m
    m._lib.load()
    return m


@pytest.fixture(scope="session")
def gpu(lib):
    lib.init(0)
    return lib


@pytest.fixture(scope="session")
def oracle_cls():
    from oracle.oracle import Oracle, build_oracle
    if not os.path.exists(os.path.join(ROOT, "oracle", "liborc.so")):
        build_oracle()
    return Oracle


_LINK_CACHE = {}


def hisq_setup(lib, oracle_cls, dims, seed=11, a=0.3, eps_naik=(0.0,)):
    """Thin links (phased), oracle HISQ links; cached per (dims, seed)."""
    key = (tuple(dims), seed, a, tuple(eps_naik))
    if key not in _LINK_CACHE:
        U = lib.apply_phases(dims, lib.gen_thin_links(dims, seed, a))
        orc = oracle_cls(dims)
        L = orc.hisq_links(U, eps_naik)
        _LINK_CACHE[key] = (U, orc, L)
    return _LINK_CACHE[key]
