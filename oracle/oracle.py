"""ctypes front end of the CPU oracle (oracle/rbffd_oracle.c).  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use
this module, as the checker.  The product path (the CUDA library behind include/rbffd.h)
never imports it.

The C file restates RadialBasisFiniteDifferences.jl's operator generation; see its
header for the reference file:line each routine follows and for how parity is pinned.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librbffd_oracle.so")

# Operator codes, identical to the CUDA library's (include/rbffd.h RBFFD_OP_*).
OPS = {"E": 0, "Dx": 1, "Dy": 2, "Dxx": 3, "Dyy": 4, "Dxy": 5, "Lap": 6, "Dxk": 7, "Dyk": 8, "HV": 9}
ORC_ESINGULAR = 3

_lib = None
_all_threads = None  # OpenMP threads of the host, read before any call narrows them


def build(force=False):
    """Compile the oracle with the Makefile beside this file."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
        os.path.join(HERE, "rbffd_oracle.c")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i64, i32 = ctypes.c_int64, ctypes.c_int
        L.orc_knn.argtypes = [P, i64, P, i64, i32, P, P, P, P, i32]
        L.orc_knn_brute.argtypes = [P, i64, P, i64, i32, P, P, P, P]
        L.orc_generate.argtypes = [P, i64, P, i64, i32, i32, i32, P, i32, P, i32, i32, P, P, P, P, P, i32]
        L.orc_generate_unscaled.argtypes = [P, i64, i32, i32, i32, i32, P, i32, i32, P, P, P, i32]
        L.orc_to_csc.argtypes = [i64, i64, i32, P, P, P, P, P]
        L.orc_spmv_rows.argtypes = [i64, i32, P, P, P, P, i32]
        L.orc_spmv_rows.restype = None
        L.orc_spmv_csc.argtypes = [i64, i64, P, P, P, P, P]
        L.orc_spmv_csc.restype = None
        L.orc_phi.argtypes = [i32, i32, i32, ctypes.c_double, ctypes.c_double]
        L.orc_phi.restype = ctypes.c_double
        L.orc_process_mesh.argtypes = [P, i64, P, i64, P, i64, P, P, P, P]
        L.orc_max_threads.restype = i32
        global _all_threads
        _all_threads = L.orc_max_threads()
        _lib = L
    return _lib


def _threads(nthreads):
    """The thread count a call runs with: nthreads, or all host threads when 0 (the C side
    keeps the last count it was given, so 0 is passed on as an explicit count)."""
    lib()
    return int(nthreads) if nthreads else _all_threads


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _pts(X):
    return np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1, 2))


def _cls(c):
    return None if c is None else np.ascontiguousarray(c, dtype=np.int32)


def _ops(ops):
    return np.array([OPS[o] if isinstance(o, str) else int(o) for o in ops], dtype=np.int32)


class OracleError(RuntimeError):
    def __init__(self, code, what, bad=-1):
        super().__init__(f"oracle {what} failed with code {code}" + (f" (node {bad})" if bad >= 0 else ""))
        self.code = code
        self.bad_node = bad


def max_threads():
    """OpenMP threads of the host (all of them, whatever a previous call narrowed them to)."""
    lib()
    return _all_threads


def knn(X, Q, k, cls_x=None, cls_q=None, nthreads=0, brute=False):
    """Exact kNN (0-based ids, (d^2, id) order) of Q among X; returns (idx, d2)."""
    X, Q = _pts(X), _pts(Q)
    cls_x, cls_q = _cls(cls_x), _cls(cls_q)
    idx = np.empty((len(Q), k), np.int32)
    d2 = np.empty((len(Q), k), np.float64)
    if brute:
        rc = lib().orc_knn_brute(_p(X), len(X), _p(Q), len(Q), k, _p(cls_x), _p(cls_q), _p(idx), _p(d2))
    else:
        rc = lib().orc_knn(_p(X), len(X), _p(Q), len(Q), k, _p(cls_x), _p(cls_q), _p(idx), _p(d2), _threads(nthreads))
    if rc:
        raise OracleError(rc, "knn")
    return idx, d2


def generate(X, Y, p, n, deg, ops, cls=None, k_deriv=0, use_inverse=True, nthreads=0):
    """Row-stencil form of generate_operator / hyperviscosity_operator.

    Returns dict(nbr=N x n stencils (rows of unused nodes are -1), nn=M nearest X ids,
    cols=M x n column ids, W=nops x M x n weights), all 0-based."""
    X, Y = _pts(X), _pts(Y)
    opv = _ops(ops)
    N, M = len(X), len(Y)
    nbr = np.full((N, n), -1, np.int32)
    nn = np.empty(M, np.int32)
    cols = np.empty((M, n), np.int32)
    W = np.empty((len(opv), M, n), np.float64)
    bad = ctypes.c_int64(-1)
    rc = lib().orc_generate(
        _p(X), N, _p(Y), M, p, n, deg, _p(_cls(cls)), len(opv), _p(opv), k_deriv, int(use_inverse),
        _p(nbr), _p(nn), _p(cols), _p(W), ctypes.byref(bad), _threads(nthreads),
    )
    if rc:
        raise OracleError(rc, "generate", bad.value)
    return dict(nbr=nbr, nn=nn, cols=cols, W=W)


def generate_unscaled(X, p, n, deg, ops, k_deriv=0, use_inverse=True, nthreads=0):
    """The collocated unscaled overloads generate_operator(X, p, n, polydeg) and
    hyperviscosity_operator(k, X, p, n, polydeg); returns dict(cols, W)."""
    X = _pts(X)
    opv = _ops(ops)
    N = len(X)
    cols = np.empty((N, n), np.int32)
    W = np.empty((len(opv), N, n), np.float64)
    bad = ctypes.c_int64(-1)
    rc = lib().orc_generate_unscaled(
        _p(X), N, p, n, deg, len(opv), _p(opv), k_deriv, int(use_inverse), _p(cols), _p(W),
        ctypes.byref(bad), _threads(nthreads),
    )
    if rc:
        raise OracleError(rc, "generate_unscaled", bad.value)
    return dict(cols=cols, W=W)


def to_csc(M, N, cols, W):
    """sparse(I, J, V): 1-based CSC (colptr, rowval, nzval) of one operator."""
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    W = np.ascontiguousarray(W, dtype=np.float64)
    n = cols.shape[1]
    colptr = np.empty(N + 1, np.int64)
    rowval = np.empty(M * n, np.int64)
    nzval = np.empty(M * n, np.float64)
    rc = lib().orc_to_csc(M, N, n, _p(cols), _p(W), _p(colptr), _p(rowval), _p(nzval))
    if rc:
        raise OracleError(rc, "to_csc")
    return colptr, rowval, nzval


def spmv_rows(cols, W, x, nthreads=0):
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    W = np.ascontiguousarray(W, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(cols.shape[0], np.float64)
    lib().orc_spmv_rows(cols.shape[0], cols.shape[1], _p(cols), _p(W), _p(x), _p(y), _threads(nthreads))
    return y


def spmv_csc(M, colptr, rowval, nzval, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(M, np.float64)
    lib().orc_spmv_csc(M, len(colptr) - 1, _p(colptr), _p(rowval), _p(nzval), _p(x), _p(y))
    return y


def phi(p, a, b, x, y):
    return lib().orc_phi(p, a, b, float(x), float(y))


def process_mesh(V, tri, bc):
    """processmesh after the file reads (oracle/rbffd_oracle.c orc_process_mesh): V (nv, 2)
    vertices, tri (ntri, 3) and bc (nbc, 2) 1-based vertex ids.  Returns (Y, normals,
    tangents, offset): Y stacks the centroids, the boundary midpoints and the ghost nodes."""
    V = np.ascontiguousarray(V, dtype=np.float64)
    tri = np.ascontiguousarray(tri, dtype=np.int64)
    bc = np.ascontiguousarray(bc, dtype=np.int64)
    ntri, nbc = len(tri), len(bc)
    Y = np.empty((ntri + 2 * nbc, 2))
    nrm, tng = np.empty((nbc, 2)), np.empty((nbc, 2))
    off = ctypes.c_double()
    rc = lib().orc_process_mesh(_p(V), len(V), _p(tri), ntri, _p(bc), nbc, _p(Y), _p(nrm), _p(tng), ctypes.byref(off))
    if rc:
        raise OracleError(rc, "orc_process_mesh")
    return Y, nrm, tng, off.value
