"""CPU accuracy check of the fixed-point r^3 routine used by the mixed-precision weight solve
(csrc/phi_fixed.cuh; host build in tests/phi_fixed_host.cpp).

The routine must return, for every node pair, the exact r^3 (and r^2) of the 61-bit
fixed-point coordinates to within one unit in the last place; its host build uses a square
root seed perturbed by up to 2^-20 so that the hardware approximation's error is covered.
The reference evaluates phi = r^3 in FP64 (src/rbfbasis.jl:9-30 via src/rbfblock.jl:1-23);
that value is also compared (a few ulps apart: it rounds dx, dy, r^2, sqrt and the cube).
"""
import ctypes
import math
import os
import shutil
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tempfile.mkdtemp(prefix="fx_")
    so = os.path.join(d, "libfx.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "phi_fixed_host.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P = ctypes.c_void_p
    lib.fx_to_fixed61.argtypes = [P, ctypes.c_int64, P]
    lib.fx_r3.argtypes = [P, ctypes.c_int64, P, P]
    yield lib
    shutil.rmtree(d, ignore_errors=True)


def to_fixed(lib, x):
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty(len(x), np.int64)
    lib.fx_to_fixed61(x.ctypes.data, len(x), out.ctypes.data)
    return out


def r3_r2(lib, pts):
    pts = np.ascontiguousarray(pts, np.float64)
    n = len(pts)
    r3 = np.empty(n)
    r2 = np.empty(n)
    lib.fx_r3(pts.ctypes.data, n, r3.ctypes.data, r2.ctypes.data)
    return r3, r2


def exact_fixed(x):
    v = Fraction(float(x)) * (1 << 61)
    return int(v) if v >= 0 else -int(-v)  # toward zero


def exact_r3_r2(fxi, fyi, fxj, fyj):
    """Correctly rounded r^3 and r^2 of fixed-point coordinates (units 2^-61)."""
    R = (fxi - fxj) ** 2 + (fyi - fyj) ** 2  # r^2 = R 2^-122
    if R == 0:
        return 0.0, 0.0
    g = 80
    s = math.isqrt(R ** 3 << (2 * g))  # floor(R^1.5 2^g)
    return float(Fraction(s, 1 << (183 + g))), float(Fraction(R, 1 << 122))


def ulps(a, b):
    ia = np.asarray(a, np.float64).view(np.int64)
    ib = np.asarray(b, np.float64).view(np.int64)
    return np.abs(ia - ib)


def sample_points(rng, n):
    """Stencil-like scaled coordinates plus edge cases."""
    pts = rng.uniform(-1.0, 1.0, (n, 4))
    k = n // 8
    pts[:k, 0] = pts[:k, 2] + rng.uniform(-1e-6, 1e-6, k)  # nearly equal x
    pts[k:2 * k, 1] = pts[k:2 * k, 3]  # equal y
    tiny = rng.uniform(-1.0, 1.0, (k, 4)) * 10.0 ** rng.uniform(-12, -2, (k, 4))
    pts[2 * k:3 * k] = tiny  # all coordinates tiny
    pts[3 * k:4 * k] = np.sign(pts[3 * k:4 * k]) * (1.0 + rng.integers(0, 4, (k, 4)) * 2.0 ** -52)
    return pts


def test_to_fixed61_exact(fx):
    rng = np.random.default_rng(3)
    x = np.concatenate([
        rng.uniform(-1.9999, 1.9999, 4000),
        rng.uniform(-1, 1, 2000) * 10.0 ** rng.uniform(-20, 0, 2000),
        [0.0, -0.0, 1.0, -1.0, 2.0 ** -9, 2.0 ** -10, 1.0 + 2.0 ** -52, np.nextafter(2.0, 0.0), 5e-324, -2.0 ** -61],
    ])
    got = to_fixed(fx, x)
    want = np.array([exact_fixed(v) for v in x], np.int64)
    assert np.array_equal(got, want)


def test_r3_fixed_within_one_ulp(fx):
    rng = np.random.default_rng(11)
    pts = sample_points(rng, 16000)
    r3, r2 = r3_r2(fx, pts)
    F = to_fixed(fx, pts.ravel()).reshape(-1, 4)
    e3 = np.empty(len(pts))
    e2 = np.empty(len(pts))
    for k in range(len(pts)):
        e3[k], e2[k] = exact_r3_r2(*(int(v) for v in F[k]))
    assert ulps(r3, e3).max() <= 1
    assert ulps(r2, e2).max() <= 1
    # the reference's FP64 evaluation (dx, dy, r^2, sqrt, cube rounded in turn), where the
    # fixed-point coordinates are exact (|x| >= 2^-9) and r is not tiny
    big = (np.abs(pts) >= 2.0 ** -9).all(1)
    dx, dy = pts[:, 0] - pts[:, 2], pts[:, 1] - pts[:, 3]
    rr = np.sqrt(dx * dx + dy * dy)
    ref = rr * rr * rr
    sel = big & (rr > 1e-3)
    assert sel.sum() > 5000
    assert (np.abs(r3[sel] - ref[sel]) <= 8 * np.spacing(ref[sel])).all()


def test_r3_fixed_edge_cases(fx):
    pts = np.array([
        [0.0, 0.0, 0.0, 0.0],  # coincident: 0
        [0.5, -0.25, 0.5, -0.25],
        [1.0, 0.0, 0.0, 0.0],  # r = 1
        [-1.0, -1.0, 1.0, 1.0],  # r^2 = 8, largest
        [1.0 + 2.0 ** -52, 0.0, -1.0 - 2.0 ** -52, 0.0],
        [0.0, 3e-19, 0.0, 0.0],  # below fixed-point resolution: 0 or 2^-61-sized
        [0.3, 0.0, 0.3 + 2.0 ** -40, 0.0],
        [2.0 ** -9, 2.0 ** -9, -(2.0 ** -9), 0.0],
    ])
    r3, r2 = r3_r2(fx, pts)
    F = to_fixed(fx, pts.ravel()).reshape(-1, 4)
    for k in range(len(pts)):
        e3, e2 = exact_r3_r2(*(int(v) for v in F[k]))
        assert ulps(r3[k], e3) <= 1, (k, r3[k], e3)
        assert ulps(r2[k], e2) <= 1, (k, r2[k], e2)
    assert r3[0] == 0.0 and r3[1] == 0.0 and r3[2] == 1.0
