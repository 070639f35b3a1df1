"""GB300-native RBF-FD hot path with the API of RadialBasisFiniteDifferences.jl.

kNN stencil selection, batched local weight solves and sparse stencil application run as
sm_103a CUDA kernels behind the C ABI in include/rbffd.h (librbffd.so, built in-tree by
_build.build()).  This package is the Python host side over that ABI; julia/RBFFDGPU.jl is
the Julia host side.
"""
from . import _build, _native, nodesets  # noqa: F401
from ._native import RbffdError  # noqa: F401
from .operators import (  # noqa: F401
    GhostClosure,
    RK4Stepper,
    GENERATE_OPS,
    HYPERVISCOSITY_OPS,
    Handle,
    OperatorSet,
    calculateneighbors,
    default_handle,
    generate_operator,
    hyperviscosity_operator,
    node_class_from_ranges,
    processmesh_arrays,
)


def build(force=False):
    return _build.build(force=force)


def lib_path():
    return _build.LIB_PATH
