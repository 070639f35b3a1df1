"""CPU tests of the C ABI library: it builds for sm_103a, loads, exports every symbol that
include/rbffd.h declares, and fails loudly (no CPU fallback) when no GPU is usable."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def header_functions():
    txt = open(os.path.join(ROOT, "include", "rbffd.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rbffd_[a-z0-9_]+)\s*\(", txt)))


def test_library_builds_and_exports_header(pkg):
    path = pkg.build()
    assert os.path.exists(path)
    L = pkg._native.load()
    names = header_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name
    assert sorted(pkg._native.EXPORTED) == names
    assert L.rbffd_version() == 1


def test_every_translation_unit_is_built(pkg):
    """Every CUDA source of csrc/ is compiled into the library, and the library leaves no
    symbol of its own unresolved (a shared library links even when one is missing)."""
    import importlib
    import subprocess

    b = importlib.import_module(pkg.__name__ + "._build")
    on_disk = sorted(f for f in os.listdir(b.CSRC) if f.endswith(".cu"))
    assert sorted(b.SOURCES) == on_disk
    path = pkg.build()
    try:
        out = subprocess.run(["nm", "-u", "-C", path], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("nm not available")
    own = [ln for ln in out.splitlines() if re.search(r"\b(rbffd_|launch_|solve_|schur_)", ln)]
    assert not own, own


def test_no_cpu_fallback_without_gpu(pkg):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = pkg._native.load()
    h = ctypes.c_void_p()
    opt = pkg._native.Options(0, 0, 0, 0.0)
    rc = L.rbffd_create(ctypes.byref(opt), ctypes.byref(h))
    assert rc == pkg._native.ECUDA and not h.value
    assert L.rbffd_last_error(None)
    with pytest.raises(pkg.RbffdError):
        pkg.Handle()


def test_built_for_sm103a_only(pkg):
    from importlib import import_module

    b = pkg._build
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert import_module("rbffd_gb300._build").SOURCES


def test_status_strings(pkg):
    L = pkg._native.load()
    assert L.rbffd_status_string(3) == b"singular local system"
