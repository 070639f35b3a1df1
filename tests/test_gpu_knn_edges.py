"""kNN near cell edges: the ring search's FP32 stopping bound must stay a lower bound.

The kNN kernel (csrc/knn.cu) stops sweeping rings of grid cells once the current k-th
squared distance is below an FP32 bound of the distance from the query to the unsearched
cells.  The bound's terms are (R + 1) cs32 - fx, with cs32 and fx truncations of the FP64
cell size and in-cell offset, so their error is absolute (about one FP32 ulp of cs) and does
not shrink with the bound.  A query a fraction of an ulp inside the right edge of its cell,
with a node A a little farther away inside the cell and a node B just across the edge, is
where a relative-only safety margin lets the search stop at A although B is nearer.  This is
the nearest-node search of non-collocated evaluation points (knn(tree, Y, 1),
src/generate_operator.jl:47, src/calculateneighbors.jl:90-94; the search radius starts at
the query's own cell for k = 1).

The construction emulates the kernel's FP32 arithmetic on the host to place such queries;
a CPU test checks that the emulated bound without the absolute margin is fooled by them
(so the GPU test exercises the case), and the GPU test checks the library's nearest nodes
against the brute-force oracle, bit-exactly.
"""
import math
from fractions import Fraction

import numpy as np
import pytest


def trunc32(x):
    """float(x) by truncation of the mantissa (the kernels' f64_to_f32, normal range)."""
    b = np.array([x], dtype=np.float64).view(np.uint64) & np.uint64(~((1 << 29) - 1) & 0xFFFFFFFFFFFFFFFF)
    return np.float32(b.view(np.float64)[0])


def round32(fr):
    """Fraction -> float32, one rounding (the value must be exact in FP64 first)."""
    d = float(fr)
    assert Fraction(d) == fr
    return np.float32(d)


def grid_params(X):
    """Cell size and counts as the library's grid build computes them (FP64, host)."""
    x0, x1 = float(X[:, 0].min()), float(X[:, 0].max())
    y0, y1 = float(X[:, 1].min()), float(X[:, 1].max())
    w, hh = x1 - x0, y1 - y0
    N = len(X)
    area = (w if w > 0 else 1.0) * (hh if hh > 0 else 1.0)
    cs = math.sqrt(2.0 * area / N)
    nx, ny = int(w / cs) + 1, int(hh / cs) + 1
    assert nx * ny <= 4 * N + 16
    return x0, y0, cs, nx, ny


def cell_of(v, v0, cs, nmax):
    c = math.floor((v - v0) / cs)
    return min(max(c, 0), nmax - 1)


def old_bound(q, x0, y0, cs, nx, ny):
    """The squared FP32 bound b2 the ring search at R = 0 compares with, with only a relative
    2^-18 shrink (no absolute margin), emulating the kernel's FP32 steps, and the query's FP32
    cell column; b2 is None where no bound applies (the search goes on)."""
    cs32 = trunc32(cs)
    ics32 = np.float32(1.0) / cs32
    dqx, dqy = q[0] - x0, q[1] - y0
    cx = int(math.floor(np.float32(trunc32(dqx) * ics32)))
    cy = int(math.floor(np.float32(trunc32(dqy) * ics32)))
    cx, cy = min(max(cx, 0), nx - 1), min(max(cy, 0), ny - 1)
    fx = trunc32(float(Fraction(-cx) * Fraction(cs) + Fraction(dqx)))
    fy = trunc32(float(Fraction(-cy) * Fraction(cs) + Fraction(dqy)))
    terms = []
    if cx > 0:
        terms.append(fx)
    if cx < nx - 1:
        terms.append(round32(Fraction(float(cs32)) - Fraction(float(fx))))
    if cy > 0:
        terms.append(fy)
    if cy < ny - 1:
        terms.append(round32(Fraction(float(cs32)) - Fraction(float(fy))))
    bound = min(terms)
    if not bound > 0:
        return None, cx
    return float(np.float32(np.float32(bound * bound) * np.float32(1.0 - 2.0 ** -18))), cx


def edge_case(seed=31, ntarget=12):
    """Base jittered grid plus, per target, nodes A and B around a query q on one row:
    A -- q | B with the cell edge at |, d(q, B) < d(q, A), both a fraction of an FP32 ulp of
    the cell size.  Returns X, Y (the queries), the number of base nodes and the number of
    targets whose emulated relative-only bound stops at A."""
    nb = 64
    rng = np.random.default_rng(seed)
    h = 1.0 / nb
    g = (np.arange(nb) + 0.5) * h
    base = np.stack(np.meshgrid(g, g), -1).reshape(-1, 2) + rng.uniform(-0.3 * h, 0.3 * h, (nb * nb, 2))
    # the planted nodes lie inside the base's bounding box, so the grid of the final set is
    # the base's box cut with the cell size of N = base + 2 ntarget nodes
    N = len(base) + 2 * ntarget
    x0, y0 = float(base[:, 0].min()), float(base[:, 1].min())
    w, hh = float(base[:, 0].max()) - x0, float(base[:, 1].max()) - y0
    cs = math.sqrt(2.0 * (w * hh) / N)
    nx, ny = int(w / cs) + 1, int(hh / cs) + 1
    u = 2.0 ** (math.floor(math.log2(cs)) - 23)  # FP32 ulp of the cell size
    eps_c = cs - float(trunc32(cs))
    A, B, Q = [], [], []
    fooled = 0
    for rr in range(3, ny - 3, 3):
        if len(Q) == ntarget:
            break
        for c in range(3, nx - 3):
            qy = y0 + (rr + 0.5) * cs
            xe = x0 + c * cs
            qx = xe - (eps_c + 0.01 * u)
            xb = xe + 0.02 * u
            if cell_of(xb, x0, cs, nx) != c or cell_of(qx, x0, cs, nx) != c - 1:
                continue
            db = xb - qx
            b2, cq = old_bound((qx, qy), x0, y0, cs, nx, ny)
            if cq != c - 1 or b2 is None or b2 <= (db * (1 + 2.0 ** -20)) ** 2:
                continue
            # A farther than B, halfway to what the relative-only bound accepts
            da = 0.5 * (db + math.sqrt(b2))
            xa = qx - da
            if cell_of(xa, x0, cs, nx) != c - 1 or not (db < qx - xa and (qx - xa) ** 2 < b2):
                continue
            # no base node may be as close to the query as A
            if np.sqrt(((base - (qx, qy)) ** 2).sum(1)).min() <= da:
                continue
            fooled += 1
            A.append((xa, qy))
            B.append((xb, qy))
            Q.append((qx, qy))
            break
    assert len(Q) == ntarget, "the cell size was computed for ntarget planted pairs"
    X = np.vstack([base, np.array(A), np.array(B)])
    assert grid_params(X) == (x0, y0, cs, nx, ny)
    return X, np.array(Q), len(base), fooled


def test_edge_construction_fools_relative_only_bound():
    """Host check: every planted query sits where a bound without the absolute margin stops at
    A although B (across the cell edge) is nearer."""
    X, Y, nbase, fooled = edge_case()
    nt = len(Y)
    assert fooled == nt == 12
    A, B = X[nbase:nbase + nt], X[nbase + nt:]
    dA = np.abs(Y[:, 0] - A[:, 0])
    dB = np.abs(B[:, 0] - Y[:, 0])
    assert (dB < dA).all()


@pytest.mark.gpu
def test_nearest_node_across_cell_edge(pkg, orc, gpu):
    """knn(tree, Y, 1) of the planted queries: the library's nearest node is B, bit-exactly
    as the brute-force oracle finds it, for every query (and for every node's own stencils)."""
    X, Y, nbase, fooled = edge_case()
    nt = len(Y)
    ix, iy, dx, dy = pkg.calculateneighbors(X, Y, 4)
    ref_y, ref_d2 = orc.knn(X, Y, 1, brute=True)
    assert np.array_equal(iy[:, 0] - 1, ref_y[:, 0])
    assert np.array_equal(iy[:, 0] - 1, nbase + nt + np.arange(nt))  # B of every target
    assert np.array_equal(dy[:, 0], np.sqrt(ref_d2[:, 0]))
    ref_x, _ = orc.knn(X, X, 4, brute=True)
    assert np.array_equal(ix - 1, ref_x)
