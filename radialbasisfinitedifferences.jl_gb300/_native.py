"""ctypes binding of librbffd.so (the C ABI declared in include/rbffd.h).

This is the same binding a Python caller of the C ABI writes; the Julia shim in
julia/RBFFDGPU.jl binds the same symbols with ccall.  There is no fallback: if the
library is missing, or no sm_103a GPU is usable, calls raise.
"""
import ctypes
import os

from . import _build

OK, EINVAL, ECUDA, ESINGULAR, ETIMEOUT, ENOMEM = 0, 1, 2, 3, 4, 5
OP_CODES = {"E": 0, "Dx": 1, "Dy": 2, "Dxx": 3, "Dyy": 4, "Dxy": 5, "Lap": 6, "Dxk": 7, "Dyk": 8, "HV": 9}
PREC = {"fp64": 0, "mixed": 1}
MEM_HOST, MEM_DEVICE = 0, 1

# Every symbol include/rbffd.h declares.
EXPORTED = [
    "rbffd_version",
    "rbffd_status_string",
    "rbffd_create",
    "rbffd_destroy",
    "rbffd_last_error",
    "rbffd_autotune_report",
    "rbffd_stream",
    "rbffd_synchronize",
    "rbffd_generate_operator",
    "rbffd_hyperviscosity_operator",
    "rbffd_generate_operator_unscaled",
    "rbffd_calculateneighbors",
    "rbffd_process_mesh",
    "rbffd_opset_create",
    "rbffd_opset_destroy",
    "rbffd_opset_shape",
    "rbffd_opset_device_csr",
    "rbffd_opset_export_csc",
    "rbffd_opset_export_csr",
    "rbffd_opset_export_stencils",
    "rbffd_spmv",
    "rbffd_spmm",
    "rbffd_rk4_create",
    "rbffd_rk4_run",
    "rbffd_rk4_apply",
    "rbffd_rk4_destroy",
    "rbffd_ghost_create",
    "rbffd_ghost_apply",
    "rbffd_ghost_destroy",
    "rbffd_rk4_set_closure",
    "rbffd_lsq_cgls",
    "rbffd_knn_noalloc",
    "rbffd_measure_fma_peaks",
]


class Options(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int),
        ("warps_per_block", ctypes.c_int),
        ("max_refine", ctypes.c_int),
        ("refine_tol", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("ms_upload", ctypes.c_double),
        ("ms_grid", ctypes.c_double),
        ("ms_knn", ctypes.c_double),
        ("ms_solve", ctypes.c_double),
        ("ms_fallback", ctypes.c_double),
        ("ms_csr", ctypes.c_double),
        ("ms_total", ctypes.c_double),
        ("n_systems", ctypes.c_int64),
        ("n_rows", ctypes.c_int64),
        ("n_fallback", ctypes.c_int64),
        ("first_bad_node", ctypes.c_int64),
        ("refine_hist", ctypes.c_int64 * 8),
        ("nnz", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "refine_hist"}
        d["refine_hist"] = list(self.refine_hist)
        return d


class LsqInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("relres", ctypes.c_double), ("ms", ctypes.c_double)]


class CSC(ctypes.Structure):
    _fields_ = [
        ("colptr", ctypes.c_void_p),
        ("rowval", ctypes.c_void_p),
        ("nzval", ctypes.c_void_p),
    ]


class Problem(ctypes.Structure):
    _fields_ = [
        ("X", ctypes.c_void_p),
        ("N", ctypes.c_int64),
        ("Y", ctypes.c_void_p),
        ("M", ctypes.c_int64),
        ("p", ctypes.c_int),
        ("n", ctypes.c_int),
        ("polydeg", ctypes.c_int),
        ("node_class", ctypes.c_void_p),
        ("n_per_node", ctypes.c_void_p),
        ("deg_per_node", ctypes.c_void_p),
        ("op_mask", ctypes.c_uint32),
        ("k_deriv", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("memspace", ctypes.c_int),
        ("row_begin", ctypes.c_int64),
        ("row_end", ctypes.c_int64),
    ]


class RbffdError(RuntimeError):
    def __init__(self, code, msg, first_bad_node=-1):
        super().__init__(f"rbffd error {code} ({_STATUS.get(code, '?')}): {msg}")
        self.code = code
        self.first_bad_node = first_bad_node


_STATUS = {0: "ok", 1: "EINVAL", 2: "ECUDA", 3: "ESINGULAR", 4: "ETIMEOUT", 5: "ENOMEM"}
_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=False):
    """Load librbffd.so.  Raises if it is missing (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("RBFFD_LIB") or _build.LIB_PATH  # RBFFD_LIB: another build of the library
    if build_if_missing and not os.path.exists(path):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"librbffd.so not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    P, i32, i64, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32
    sig = {
        "rbffd_version": ([], i32),
        "rbffd_status_string": ([i32], ctypes.c_char_p),
        "rbffd_create": ([P, P], i32),
        "rbffd_destroy": ([P], None),
        "rbffd_last_error": ([P], ctypes.c_char_p),
        "rbffd_autotune_report": ([P], ctypes.c_char_p),
        "rbffd_stream": ([P], P),
        "rbffd_synchronize": ([P], i32),
        "rbffd_generate_operator": ([P, P, i64, P, i64, i32, i32, i32, P, u32, i32, P, P], i32),
        "rbffd_hyperviscosity_operator": ([P, i32, P, i64, P, i64, i32, i32, i32, P, i32, P, P], i32),
        "rbffd_generate_operator_unscaled": ([P, P, i64, i32, i32, i32, u32, i32, P, P], i32),
        "rbffd_calculateneighbors": ([P, P, i64, P, i64, i32, P, P, P, P, P], i32),
        "rbffd_process_mesh": ([P, P, i64, P, i64, P, i64, P, P, P, P], i32),
        "rbffd_opset_create": ([P, P, P, P], i32),
        "rbffd_opset_destroy": ([P, P], None),
        "rbffd_opset_shape": ([P, P, P, P, P], i32),
        "rbffd_opset_device_csr": ([P, i32, P, P, P], i32),
        "rbffd_opset_export_csc": ([P, P, i32, P], i32),
        "rbffd_opset_export_csr": ([P, P, i32, P, P, P], i32),
        "rbffd_opset_export_stencils": ([P, P, P, P], i32),
        "rbffd_spmv": ([P, P, i32, P, P], i32),
        "rbffd_spmm": ([P, P, i32, P, P, i32, i32], i32),
        "rbffd_rk4_create": ([P, P, i32, P, P, i32, i32, P], i32),
        "rbffd_rk4_run": ([P, P, P, ctypes.c_double, i64], i32),
        "rbffd_rk4_apply": ([P, P, P, P], i32),
        "rbffd_rk4_destroy": ([P, P], None),
        "rbffd_ghost_create": ([P, P, i32, P, P, i64, P], i32),
        "rbffd_ghost_apply": ([P, P, P, i32, i32], i32),
        "rbffd_ghost_destroy": ([P, P], None),
        "rbffd_rk4_set_closure": ([P, P, P, i32], i32),
        "rbffd_lsq_cgls": ([P, P, P, P, P, i64, ctypes.c_double, P], i32),
        "rbffd_knn_noalloc": ([P, i64, i32, P, P, P], i32),
        "rbffd_measure_fma_peaks": ([i32, P, P], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(h, rc, stats=None):
    if rc != OK:
        msg = load().rbffd_last_error(h)
        bad = stats.first_bad_node if stats is not None else -1
        raise RbffdError(rc, msg.decode() if msg else "", bad)
