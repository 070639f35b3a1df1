import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden", "tominec_fitted.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and librbffd.so")


@pytest.fixture(scope="session")
def pkg():
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def tominec():
    g = np.load(GOLDEN)
    return {k: g[k] for k in g.files}


@pytest.fixture(scope="session")
def gpu(pkg):
    """The built library and a handle on cuda:0 (GPU tests only)."""
    pkg.build()
    return pkg.default_handle()


def rel_row_err(W, Wref):
    """max over rows of ||w_i - w_i^ref||_inf / ||w_i^ref||_inf"""
    W = np.asarray(W).reshape(Wref.shape)
    return float((np.abs(W - Wref).max(-1) / np.abs(Wref).max(-1)).max())
