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


def rect_tri_mesh(nx, ny, seed, jitter=0.25, reverse=False):
    """A triangulated unit square as a CGNS mesh would hold it (for processmesh): vertices
    (interior ones jittered by up to jitter * h), 1-based triangles (two per cell) and four
    boundary markers (bottom, right, top, left) of 1-based line elements, listed
    counter-clockwise around the domain (clockwise when reverse)."""
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.linspace(0.0, 1.0, nx + 1), np.linspace(0.0, 1.0, ny + 1))
    V = np.stack([xs.ravel(), ys.ravel()], axis=1)
    inner = (V[:, 0] > 0) & (V[:, 0] < 1) & (V[:, 1] > 0) & (V[:, 1] < 1)
    V[inner] += rng.uniform(-jitter, jitter, (int(inner.sum()), 2)) * np.array([1.0 / nx, 1.0 / ny])

    def v(i, j):
        return j * (nx + 1) + i + 1

    tri = []
    for j in range(ny):
        for i in range(nx):
            tri.append((v(i, j), v(i + 1, j), v(i + 1, j + 1)))
            tri.append((v(i, j), v(i + 1, j + 1), v(i, j + 1)))
    bottom = [(v(i, 0), v(i + 1, 0)) for i in range(nx)]
    right = [(v(nx, j), v(nx, j + 1)) for j in range(ny)]
    top = [(v(i + 1, ny), v(i, ny)) for i in reversed(range(nx))]
    left = [(v(0, j + 1), v(0, j)) for j in reversed(range(ny))]
    markers = [np.array(m, np.int64) for m in (bottom, right, top, left)]
    if reverse:
        markers = [m[:, ::-1].copy() for m in markers]
    return V, np.array(tri, np.int64), markers
