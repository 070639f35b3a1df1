"""Independent numpy/scipy restatement of the reference's operator generation.
TEST INFRASTRUCTURE ONLY (CPU tests cross-check the C oracle with it at small N).

It shares no code with oracle/rbffd_oracle.c:
  - kNN: scipy.spatial.cKDTree (the reference uses NearestNeighbors.jl KDTree,
    src/generate_operator.jl:43-47);
  - phi derivatives: symbolic differentiation of sqrt(x^2+y^2)^p with sympy, the way
    src/rbfbasis.jl:9-30 and src/rbfbasis_k.jl:9-20 use Symbolics;
  - local systems: batched numpy.linalg.inv of [Phi P; P' 0] (src/interpolationmatrix.jl:3-8)
    times the RHS, rows 1..n kept and unscaled (src/generate_operator.jl:89-167).
The polynomial basis here is ordered differently from the C oracle (x-powers first), which
exercises the fact that the weights do not depend on the basis order.
"""
import functools

import numpy as np
import scipy.spatial

EPS = np.finfo(np.float64).eps

# (a, b) derivative orders of each operator; combined operators have two terms.
_OPS = {
    "E": [(0, 0)], "Dx": [(1, 0)], "Dy": [(0, 1)], "Dxx": [(2, 0)], "Dyy": [(0, 2)],
    "Dxy": [(1, 1)], "Lap": [(2, 0), (0, 2)],
}


@functools.lru_cache(maxsize=None)
def _phi_fn(p, a, b):
    import sympy

    x, y = sympy.symbols("x y", real=True)
    e = sympy.sqrt(x**2 + y**2) ** p
    if a:
        e = sympy.diff(e, x, a)
    if b:
        e = sympy.diff(e, y, b)
    return sympy.lambdify((x, y), e, "numpy")


def _monos(d):
    return [(a, t - a) for t in range(d + 1) for a in range(0, t + 1)]


def _op_terms(op, K):
    if op == "Dxk":
        return [(K, 0)]
    if op == "Dyk":
        return [(0, K)]
    if op == "HV":
        return [(K, 0), (0, K)]
    return _OPS[op]


def _falling(e, k):
    c = np.ones_like(e, dtype=np.float64)
    for t in range(k):
        c = c * (e - t)
    return c


def generate(X, Y, p, n, deg, ops, k_deriv=0):
    """Returns (cols M x n, W nops x M x n) of generate_operator(X, Y, p, n, deg)."""
    X = np.asarray(X, np.float64).reshape(-1, 2)
    Y = np.asarray(Y, np.float64).reshape(-1, 2)
    tree = scipy.spatial.cKDTree(X)
    _, nbr = tree.query(X, n)
    _, nn = tree.query(Y, 1)
    nn = np.asarray(nn).reshape(-1)
    st = nbr[nn]  # stencil of the nearest X node of each Y point
    Xl = X[st]  # M x n x 2
    xc = X[nn][:, None, :]
    Xd = Xl - xc
    scale = 1.0 / np.abs(Xd).max(axis=1)  # M x 2, src/scalestencil.jl:17-18
    Xs = Xd * scale[:, None, :]
    D = Xs[:, :, None, :] - Xs[:, None, :, :]
    Phi = _phi_fn(p, 0, 0)(D[..., 0], D[..., 1])
    monos = _monos(deg)
    m = len(monos)
    P = np.stack([Xs[..., 0] ** a * Xs[..., 1] ** b for a, b in monos], -1)  # M x n x m
    Mn = len(Y)
    A = np.zeros((Mn, n + m, n + m))
    A[:, :n, :n] = Phi
    A[:, :n, n:] = P
    A[:, n:, :n] = np.transpose(P, (0, 2, 1))
    Ainv = np.linalg.inv(A)
    ys = (Y - X[nn]) * scale  # src/generate_operator.jl:110,120
    sc = ys[:, None, :] - Xs
    sc = np.where(sc == 0, EPS, sc)
    W = []
    for op in ops:
        terms = _op_terms(op, k_deriv)
        rhs = np.zeros((Mn, n + m))
        for a, b in terms:
            c = scale[:, 0] ** a * scale[:, 1] ** b if len(terms) > 1 else np.ones(Mn)
            f = _phi_fn(p, a, b)
            rhs[:, :n] += c[:, None] * np.broadcast_to(f(sc[..., 0], sc[..., 1]), (Mn, n))
            for j, (ea, eb) in enumerate(monos):
                if ea >= a and eb >= b:
                    rhs[:, n + j] += c * _falling(np.float64(ea), a) * _falling(np.float64(eb), b) * (
                        ys[:, 0] ** (ea - a) * ys[:, 1] ** (eb - b)
                    )
        w = np.einsum("mij,mj->mi", Ainv[:, :n, :], rhs)
        if len(terms) == 1:
            a, b = terms[0]
            w = w * (scale[:, 0] ** a * scale[:, 1] ** b)[:, None]
        W.append(w)
    return st.astype(np.int32), np.stack(W)
