"""Host-side mirror of RadialBasisFiniteDifferences.jl's operator API over librbffd.

Same names, argument meaning and return values as the Julia package
(src/generate_operator.jl, src/hyperviscosity_operator.jl, src/calculateneighbors.jl),
with SparseMatrixCSC{Float64,Int64} returned as scipy.sparse.csc_matrix.  Index sets are
1-based like Julia's (UnitRange or integer arrays).  All arithmetic runs on the GPU through
the C ABI; nothing here computes weights on the CPU.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _native as nat

GENERATE_OPS = ("E", "Dx", "Dy", "Dxx", "Dyy", "Dxy")
HYPERVISCOSITY_OPS = ("Dxk", "Dyk")


class Handle:
    """Owns an rbffd_handle (device, CUDA stream, options)."""

    def __init__(self, device=0, warps_per_block=0, max_refine=0, refine_tol=0.0):
        self._lib = nat.load()
        opt = nat.Options(device, warps_per_block, max_refine, refine_tol)
        h = ctypes.c_void_p()
        rc = self._lib.rbffd_create(ctypes.byref(opt), ctypes.byref(h))
        if rc != nat.OK:
            msg = self._lib.rbffd_last_error(None)
            raise nat.RbffdError(rc, msg.decode() if msg else "rbffd_create failed")
        self.ptr = h

    @property
    def stream(self):
        return self._lib.rbffd_stream(self.ptr)

    def synchronize(self):
        nat.check(self.ptr, self._lib.rbffd_synchronize(self.ptr))

    def autotune_report(self):
        """The solve autotuner's per-class choices on this handle (rbffd_autotune_report)."""
        r = self._lib.rbffd_autotune_report(self.ptr)
        return [ln for ln in (r.decode() if r else "").splitlines() if ln]

    def close(self):
        if self.ptr:
            self._lib.rbffd_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_handle = None


def default_handle():
    global _default_handle
    if _default_handle is None:
        _default_handle = Handle()
    return _default_handle


def _pts(X):
    a = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1, 2))
    if a.size == 0:
        raise ValueError("empty point set")
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _ids(r):
    return np.asarray(list(r) if isinstance(r, range) else r, dtype=np.int64).reshape(-1)


def node_class_from_ranges(N, X_idx_in, X_idx_bc, X_idx_bc_g):
    """Class of every node from the index ranges of calculateneighbors
    (src/calculateneighbors.jl:1-2): 0 interior, +b boundary b, -b ghost of b (1-based ids)."""
    cls = np.full(N, np.iinfo(np.int32).min, dtype=np.int32)
    cls[_ids(X_idx_in) - 1] = 0
    for b, r in enumerate(X_idx_bc, start=1):
        cls[_ids(r) - 1] = b
    for b, r in enumerate(X_idx_bc_g, start=1):
        cls[_ids(r) - 1] = -b
    if (cls == np.iinfo(np.int32).min).any():
        raise ValueError("every node must be in X_idx_in, X_idx_bc or X_idx_bc_g")
    return cls


def _mask(ops):
    m = 0
    for o in ops:
        m |= 1 << nat.OP_CODES[o]
    return m


def _ordered(ops):
    """ops in the library's output order (increasing operator code)."""
    return sorted(ops, key=lambda o: nat.OP_CODES[o])


def _alloc_csc(M, N, nnz, nops):
    bufs = []
    arr = (nat.CSC * nops)()
    for q in range(nops):
        colptr = np.empty(N + 1, np.int64)
        rowval = np.empty(nnz, np.int64)
        nzval = np.empty(nnz, np.float64)
        arr[q].colptr = colptr.ctypes.data
        arr[q].rowval = rowval.ctypes.data
        arr[q].nzval = nzval.ctypes.data
        bufs.append((colptr, rowval, nzval))
    return arr, bufs


def _to_scipy(M, N, colptr, rowval, nzval):
    # Julia's SparseMatrixCSC arrays are 1-based
    return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(M, N))


def _finish(bufs, M, N, ops, want, stats, return_stats):
    mats = {o: _to_scipy(M, N, *b) for o, b in zip(ops, bufs)}
    out = tuple(mats[o] for o in want)
    return (out, stats.as_dict()) if return_stats else out


def generate_operator(X, *args, precision="fp64", handle=None, ops=None, return_stats=False):
    """generate_operator(X, Y, p, n, polydeg) -> (E, Dx, Dy, Dxx, Dyy, Dxy)
    (src/generate_operator.jl:29-190);
    generate_operator(X, Y, p, n, polydeg, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc,
    Y_idx_bc_g) (:192-352); generate_operator(X, p, n, polydeg) (:354-491).

    `ops` selects other operators (any of E, Dx, Dy, Dxx, Dyy, Dxy, Lap), returned in the
    order given.  `precision` is "fp64" or "mixed"."""
    h = handle or default_handle()
    L = nat.load()
    same = len(args) >= 4 and args[0] is X
    X = _pts(X)
    N = len(X)
    want = tuple(ops) if ops is not None else GENERATE_OPS
    order = _ordered(set(want))
    stats = nat.Stats()
    if len(args) == 3:
        p, n, polydeg = args
        M = N
        arr, bufs = _alloc_csc(M, N, M * n, len(order))
        rc = L.rbffd_generate_operator_unscaled(h.ptr, _ptr(X), N, p, n, polydeg, _mask(order), 0, arr,
                                                ctypes.byref(stats))
        nat.check(h.ptr, rc, stats)
        return _finish(bufs, M, N, order, want, stats, return_stats)
    if len(args) not in (4, 10):
        raise TypeError("generate_operator(X, Y, p, n, polydeg[, 6 index ranges]) or (X, p, n, polydeg)")
    Y, p, n, polydeg = args[:4]
    cls = node_class_from_ranges(N, *args[4:7]) if len(args) == 10 else None
    Y = X if same else _pts(Y)
    M = len(Y)
    arr, bufs = _alloc_csc(M, N, M * n, len(order))
    rc = L.rbffd_generate_operator(h.ptr, _ptr(X), N, _ptr(Y), M, p, n, polydeg, _ptr(cls), _mask(order),
                                   nat.PREC[precision], arr, ctypes.byref(stats))
    nat.check(h.ptr, rc, stats)
    return _finish(bufs, M, N, order, want, stats, return_stats)


def hyperviscosity_operator(k_deriv, X, *args, precision="fp64", handle=None, return_stats=False):
    """hyperviscosity_operator(k_deriv, X, Y, p, n, polydeg[, 6 index ranges]) -> (Dxk, Dyk)
    (src/hyperviscosity_operator.jl:26-175, :177-312); hyperviscosity_operator(k, X, p, n,
    polydeg) (:314-440)."""
    h = handle or default_handle()
    L = nat.load()
    same = len(args) >= 4 and args[0] is X
    X = _pts(X)
    N = len(X)
    stats = nat.Stats()
    if len(args) == 3:
        p, n, polydeg = args
        arr, bufs = _alloc_csc(N, N, N * n, 2)
        rc = L.rbffd_generate_operator_unscaled(h.ptr, _ptr(X), N, p, n, polydeg,
                                                _mask(HYPERVISCOSITY_OPS), k_deriv, arr, ctypes.byref(stats))
        nat.check(h.ptr, rc, stats)
        return _finish(bufs, N, N, HYPERVISCOSITY_OPS, HYPERVISCOSITY_OPS, stats, return_stats)
    if len(args) not in (4, 10):
        raise TypeError("hyperviscosity_operator(k, X, Y, p, n, polydeg[, 6 index ranges]) or (k, X, p, n, polydeg)")
    Y, p, n, polydeg = args[:4]
    cls = node_class_from_ranges(N, *args[4:7]) if len(args) == 10 else None
    Y = X if same else _pts(Y)
    M = len(Y)
    arr, bufs = _alloc_csc(M, N, M * n, 2)
    rc = L.rbffd_hyperviscosity_operator(h.ptr, k_deriv, _ptr(X), N, _ptr(Y), M, p, n, polydeg, _ptr(cls),
                                         nat.PREC[precision], arr, ctypes.byref(stats))
    nat.check(h.ptr, rc, stats)
    return _finish(bufs, M, N, HYPERVISCOSITY_OPS, HYPERVISCOSITY_OPS, stats, return_stats)


def calculateneighbors(X, Y, n, X_idx_in=None, X_idx_bc=(), X_idx_bc_g=(), Y_idx_in=None, Y_idx_bc=None,
                       Y_idx_bc_g=None, handle=None):
    """calculateneighbors(X, Y, n, X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc, Y_idx_bc_g)
    -> (idxs_x, idxs_y_x, dists_x, dists_y_x) (src/calculateneighbors.jl:1-97), 1-based ids.
    With X_idx_in=None every node is interior (the plain knn of src/generate_operator.jl:43-47).
    The Y index ranges are accepted and unused, as in the reference."""
    h = handle or default_handle()
    L = nat.load()
    X = _pts(X)
    N = len(X)
    Y = _pts(Y)
    M = len(Y)
    cls = None if X_idx_in is None else node_class_from_ranges(N, X_idx_in, X_idx_bc, X_idx_bc_g)
    ix = np.empty((N, n), np.int64)
    dx = np.empty((N, n), np.float64)
    iy = np.empty((M, 1), np.int64)
    dy = np.empty((M, 1), np.float64)
    rc = L.rbffd_calculateneighbors(h.ptr, _ptr(X), N, _ptr(Y), M, n, _ptr(cls), _ptr(ix), _ptr(dx), _ptr(iy),
                                    _ptr(dy))
    nat.check(h.ptr, rc)
    return ix, iy, dx, dy


def processmesh_arrays(vertices, tri, bc_lines, handle=None):
    """processmesh(meshname, markernames) (src/processmesh.jl:1-192) after its HDF5/CGNS
    reads, on arrays: vertices (nv, 2); tri (ntri, 3) 1-based vertex ids of the triangles;
    bc_lines: one (nb_i, 2) array of 1-based vertex ids per marker, in element-range order.
    Returns (Y, Y_idx_in, Y_idx_bc, Y_idx_bc_g, bc_normals, bc_tangents, offset) as the
    reference does (1-based index ranges as Python ranges, per-marker normal and tangent
    arrays), with Y the centroids, the line midpoints and the ghost nodes."""
    h = handle or default_handle()
    L = nat.load()
    V = _pts(vertices)
    T = np.ascontiguousarray(tri, dtype=np.int64).reshape(-1, 3)
    parts = [np.ascontiguousarray(b, dtype=np.int64).reshape(-1, 2) for b in bc_lines]
    B = np.ascontiguousarray(np.concatenate(parts)) if parts else np.empty((0, 2), np.int64)
    ntri, nbc = len(T), len(B)
    Y = np.empty((ntri + 2 * nbc, 2))
    nrm, tng = np.empty((nbc, 2)), np.empty((nbc, 2))
    off = ctypes.c_double()
    rc = L.rbffd_process_mesh(h.ptr, _ptr(V), len(V), _ptr(T), ntri, _ptr(B), nbc, _ptr(Y), _ptr(nrm), _ptr(tng),
                              ctypes.byref(off))
    nat.check(h.ptr, rc)
    idx_bc, idx_g, normals, tangents, a = [], [], [], [], 0
    for p in parts:
        idx_bc.append(range(ntri + a + 1, ntri + a + len(p) + 1))
        idx_g.append(range(ntri + nbc + a + 1, ntri + nbc + a + len(p) + 1))
        normals.append(nrm[a:a + len(p)])
        tangents.append(tng[a:a + len(p)])
        a += len(p)
    return Y, range(1, ntri + 1), idx_bc, idx_g, normals, tangents, off.value


class GhostClosure:
    """Ghost-node closure of one boundary (rbffd_ghost_*): u[G] = -inv(A[B,G]) A[B,~G] u with A
    one operator of a collocated set, B the boundary nodes and G their ghosts
    (examples/adv_diff_test.jl:108-141, 160-176)."""

    def __init__(self, opset, op, bnodes, gnodes, handle=None):
        self.h = handle or opset.h
        self._lib = nat.load()
        self.opset = opset
        b = np.ascontiguousarray(bnodes, dtype=np.int32)
        g = np.ascontiguousarray(gnodes, dtype=np.int32)
        if b.shape != g.shape:
            raise ValueError("one ghost per boundary node")
        out = ctypes.c_void_p()
        nat.check(self.h.ptr, self._lib.rbffd_ghost_create(self.h.ptr, opset.ptr, opset.op_index(op), _ptr(b), _ptr(g),
                                                           len(b), ctypes.byref(out)))
        self.ptr = out

    def apply(self, u):
        """u: CUDA tensor [rows, nfields] (float64 or float32), ghost rows overwritten in place."""
        import torch

        dtype = 0 if u.dtype == torch.float64 else 1
        torch.cuda.current_stream().synchronize()
        nat.check(self.h.ptr, self._lib.rbffd_ghost_apply(self.h.ptr, self.ptr, ctypes.c_void_p(u.data_ptr()),
                                                          u.shape[1] if u.dim() > 1 else 1, dtype))
        self.h.synchronize()
        return u

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.rbffd_ghost_destroy(self.h.ptr, self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RK4Stepper:
    """Explicit RK4 for du/dt = L u with L = sum_i coef[i] A_i over the operators of one or
    more OperatorSets sharing a stencil pattern (rbffd_rk4_*): the time-stepping loop of
    examples/adv_diff_test.jl:144-199 on the GPU, pairs of steps replayed as CUDA graphs."""

    def __init__(self, sets, coef, nfields, dtype="f64", fixed_rows=None, handle=None):
        self.sets = list(sets)
        self.h = handle or self.sets[0].h
        self._lib = nat.load()
        self.dtype = 0 if dtype == "f64" else 1
        arr = (ctypes.c_void_p * len(self.sets))(*[s.ptr.value for s in self.sets])
        c = np.ascontiguousarray(coef, dtype=np.float64)
        if len(c) != sum(len(s.ops) for s in self.sets):
            raise ValueError("one coefficient per operator of every set")
        fx = None if fixed_rows is None else np.ascontiguousarray(fixed_rows, dtype=np.uint8)
        out = ctypes.c_void_p()
        rc = self._lib.rbffd_rk4_create(self.h.ptr, arr, len(self.sets), _ptr(c), _ptr(fx), nfields, self.dtype,
                                        ctypes.byref(out))
        nat.check(self.h.ptr, rc)
        self.ptr = out
        self.nfields = nfields

    def set_closures(self, closures):
        """Ghost closures applied to every stage input (rbffd_rk4_set_closure)."""
        self._closures = list(closures)
        arr = (ctypes.c_void_p * max(1, len(self._closures)))(*[c.ptr.value for c in self._closures])
        nat.check(self.h.ptr, self._lib.rbffd_rk4_set_closure(self.h.ptr, self.ptr, arr, len(self._closures)))

    def run(self, u, dt, nsteps):
        """u: CUDA tensor [rows, nfields] (float64 or float32 to match dtype), advanced in place."""
        import torch

        torch.cuda.current_stream().synchronize()
        nat.check(self.h.ptr, self._lib.rbffd_rk4_run(self.h.ptr, self.ptr, ctypes.c_void_p(u.data_ptr()), dt, nsteps))
        self.h.synchronize()
        return u

    def run_ptr(self, u_ptr, dt, nsteps):
        nat.check(self.h.ptr, self._lib.rbffd_rk4_run(self.h.ptr, self.ptr, ctypes.c_void_p(u_ptr), dt, nsteps))

    def apply(self, x, y):
        import torch

        torch.cuda.current_stream().synchronize()
        nat.check(self.h.ptr, self._lib.rbffd_rk4_apply(self.h.ptr, self.ptr, ctypes.c_void_p(x.data_ptr()),
                                                        ctypes.c_void_p(y.data_ptr())))
        self.h.synchronize()
        return y

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.rbffd_rk4_destroy(self.h.ptr, self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """__cuda_array_interface__ view of library-owned device memory."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


class OperatorSet:
    """Device-resident operators of one node set (rbffd_opset): kNN + weight solves + CSR on
    the GPU, kept in HBM for stencil application (SpMV / SpMM)."""

    def __init__(self, X, Y=None, p=3, n=30, polydeg=3, ops=("Dx", "Dy", "Lap"), precision="fp64",
                 node_class=None, n_per_node=None, deg_per_node=None, k_deriv=0, row_range=None,
                 handle=None, device=False):
        """X, Y, node_class, n_per_node, deg_per_node: numpy arrays (host) or, with device=True,
        CUDA tensors (anything with .data_ptr()) already in HBM."""
        self.h = handle or default_handle()
        self._lib = nat.load()
        self.ops = tuple(_ordered(set(ops)))
        self._keep = []

        def arg(a, dtype, shape2=False):
            if a is None:
                return None, 0
            if device:
                self._keep.append(a)
                return ctypes.c_void_p(a.data_ptr()), (a.shape[0])
            arr = _pts(a) if shape2 else np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(arr)
            return _ptr(arr), len(arr)

        pX, N = arg(X, np.float64, True)
        pY, M = arg(Y, np.float64, True) if Y is not None else (None, 0)
        pc, _ = arg(node_class, np.int32)
        pn, _ = arg(n_per_node, np.int32)
        pd, _ = arg(deg_per_node, np.int32)
        rb, re = row_range if row_range is not None else (0, 0)
        prob = nat.Problem(pX, N, pY, M, p, n, polydeg, pc, pn, pd, _mask(self.ops), k_deriv,
                           nat.PREC[precision], nat.MEM_DEVICE if device else nat.MEM_HOST, rb, re)
        self.stats = nat.Stats()
        s = ctypes.c_void_p()
        rc = self._lib.rbffd_opset_create(self.h.ptr, ctypes.byref(prob), ctypes.byref(s), ctypes.byref(self.stats))
        nat.check(self.h.ptr, rc, self.stats)
        self.ptr = s
        self._keep.clear()
        rows, cols, nnz, nops = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        self._lib.rbffd_opset_shape(s, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz), ctypes.byref(nops))
        self.rows, self.cols, self.nnz = rows.value, cols.value, nnz.value
        self.row_begin = rb

    def op_index(self, op):
        return self.ops.index(op) if isinstance(op, str) else int(op)

    def csr(self, op):
        q = self.op_index(op)
        rp = np.empty(self.rows + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        nat.check(self.h.ptr, self._lib.rbffd_opset_export_csr(self.h.ptr, self.ptr, q, _ptr(rp), _ptr(col), _ptr(val)))
        return sp.csr_matrix((val, col, rp), shape=(self.rows, self.cols))

    def csr_arrays(self, op):
        """(row_ptr, col, val) exactly as stored (stencil order inside each row)."""
        m = self.csr(op)
        return m.indptr, m.indices, m.data

    def csc_julia(self, op):
        """1-based (colptr, rowval, nzval): the SparseMatrixCSC{Float64,Int64} arrays."""
        q = self.op_index(op)
        arr, bufs = _alloc_csc(self.rows, self.cols, self.nnz, 1)
        nat.check(self.h.ptr, self._lib.rbffd_opset_export_csc(self.h.ptr, self.ptr, q, arr))
        return bufs[0]

    def csc(self, op):
        cp, rv, nz = self.csc_julia(op)
        return sp.csc_matrix((nz, rv - 1, cp - 1), shape=(self.row_begin + self.rows, self.cols))

    def stencils(self):
        nbr = np.empty((self.cols, self._n_uniform()), np.int32)
        nn = np.empty(self.rows, np.int32)
        nat.check(self.h.ptr, self._lib.rbffd_opset_export_stencils(self.h.ptr, self.ptr, _ptr(nbr), _ptr(nn)))
        return nbr, nn

    def _n_uniform(self):
        return self.nnz // self.rows

    def device_csr(self, op):
        rp, col, val = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        nat.check(self.h.ptr, self._lib.rbffd_opset_device_csr(self.ptr, self.op_index(op), ctypes.byref(rp),
                                                                ctypes.byref(col), ctypes.byref(val)))
        return rp.value, col.value, val.value

    def device_values(self, op):
        """Zero-copy torch view (float64, nnz) of one operator's CSR values in HBM."""
        import torch

        _, _, val = self.device_csr(op)
        return torch.as_tensor(_DeviceArray(val, self.nnz, "<f8"), device="cuda")

    def spmv_ptr(self, op, x_ptr, y_ptr):
        """y = A_op x on the handle's stream (raw device pointers, FP64)."""
        nat.check(self.h.ptr, self._lib.rbffd_spmv(self.h.ptr, self.ptr, self.op_index(op), x_ptr, y_ptr))

    def spmm_ptr(self, op, x_ptr, y_ptr, nfields, dtype=0):
        nat.check(self.h.ptr, self._lib.rbffd_spmm(self.h.ptr, self.ptr, self.op_index(op), x_ptr, y_ptr,
                                                   nfields, dtype))

    def spmv(self, op, x, y):
        """torch CUDA tensors; ordered with torch's current stream by synchronising both sides."""
        import torch

        torch.cuda.current_stream().synchronize()
        self.spmv_ptr(op, x.data_ptr(), y.data_ptr())
        self.h.synchronize()
        return y

    def spmm(self, op, x, y):
        import torch

        dtype = 0 if x.dtype == torch.float64 else 1
        torch.cuda.current_stream().synchronize()
        self.spmm_ptr(op, x.data_ptr(), y.data_ptr(), x.shape[1], dtype)
        self.h.synchronize()
        return y

    def lsq_cgls(self, coef, f, u0=None, maxit=20000, tol=1e-12):
        """u minimising ||D u - f|| with D[i, :] = sum_q coef[q, i] A_q[i, :] (operators in set
        order), by CGLS on the GPU (rbffd_lsq_cgls): the `D \\ f` of test/poisson_test.jl.
        Returns (u, iterations, relres)."""
        c = np.ascontiguousarray(coef, dtype=np.float64)
        if c.shape != (len(self.ops), self.rows):
            raise ValueError("coef must be (number of operators, rows)")
        fv = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(self.cols) if u0 is None else np.array(u0, dtype=np.float64)
        info = nat.LsqInfo()
        nat.check(self.h.ptr, self._lib.rbffd_lsq_cgls(self.h.ptr, self.ptr, _ptr(c), _ptr(fv), _ptr(u), int(maxit),
                                                       float(tol), ctypes.byref(info)))
        return u, info.iterations, info.relres

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.rbffd_opset_destroy(self.h.ptr, self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
