"""The allocation-free kNN entry point (rbffd_knn_noalloc), called through the C ABI.

It serves callers that cannot allocate device memory: programs whose device memory belongs
to another allocator (a CUDA.jl or PyTorch caching pool), or whose memory budget is fixed at
start-up, or that must not synchronise the device the way cudaMalloc/cudaFree may.  Its
scratch is a static device array, so the test checks two calls in a row on different node
sets -- the second must not see anything the first left behind -- against the allocating
entry point rbffd_calculateneighbors (bit-exact, the bar every kNN test here uses), and the
rejection of node counts above the array's capacity.

This file is named so that pytest collects it last; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(pkg, X, k, with_d2=True):
    import torch

    L = pkg._native.load()
    Xd = torch.tensor(np.ascontiguousarray(X), dtype=torch.float64, device="cuda")
    idx = torch.full((len(X), k), -7, dtype=torch.int32, device="cuda")
    d2 = torch.full((len(X), k), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = L.rbffd_knn_noalloc(ctypes.c_void_p(Xd.data_ptr()), len(X), k, ctypes.c_void_p(idx.data_ptr()),
                             ctypes.c_void_p(d2.data_ptr()) if with_d2 else None,
                             ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    return rc, idx.cpu().numpy(), d2.cpu().numpy()


def _check(pkg, X, k, with_d2=True):
    rc, idx, d2 = _noalloc(pkg, X, k, with_d2)
    assert rc == 0, pkg._native.load().rbffd_last_error(None)
    ref_idx, _, ref_d, _ = pkg.calculateneighbors(X, X[:1], k)
    assert np.array_equal(idx.astype(np.int64) + 1, ref_idx)
    if with_d2:
        assert np.array_equal(np.sqrt(d2), ref_d)
    else:
        assert (d2 == -1.0).all()  # the distance buffer was not passed and stays untouched


def test_noalloc_matches_allocating_entry_point_twice(pkg, gpu):
    X1, _, _ = pkg.nodesets.jittered_grid(80, seed=11)            # 6400 nodes
    X2, _, _ = pkg.nodesets.jittered_grid(120, 40, seed=12)       # 4800 nodes, other shape
    for X, k in ((X1, 30), (X2, 20)):
        _check(pkg, X, k)


def test_noalloc_at_capacity(pkg, gpu):
    """Exactly RBFFD_NOALLOC_MAX_NODES = 65,536 nodes: the largest cell count the scratch holds
    (up to 2 N + 16 cells) must fit, and the result must match the allocating entry point."""
    X, _, _ = pkg.nodesets.jittered_grid(256, seed=13)
    assert len(X) == 65536
    _check(pkg, X, 30)


def test_noalloc_without_distances_and_degenerate_boxes(pkg, gpu):
    """d2_dev = NULL (indices only), and node sets whose bounding box has zero height or zero
    width (collinear nodes: one row or one column of cells)."""
    X, _, _ = pkg.nodesets.jittered_grid(60, seed=14)
    _check(pkg, X, 15, with_d2=False)
    t = np.arange(3000, dtype=np.float64) / 3000.0
    row = np.stack([t, np.full_like(t, 0.25)], 1)
    col = np.stack([np.full_like(t, -1.5), t[::-1] * 2.0], 1)
    for Xc in (row, col):
        _check(pkg, Xc, 12)


def test_noalloc_rejects_too_many_nodes(pkg, gpu):
    import torch

    L = pkg._native.load()
    n = 65536 + 1
    Xd = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    idx = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    rc = L.rbffd_knn_noalloc(ctypes.c_void_p(Xd.data_ptr()), n, 4, ctypes.c_void_p(idx.data_ptr()), None, None)
    assert rc == pkg._native.EINVAL
    assert b"65536" in L.rbffd_last_error(None)
