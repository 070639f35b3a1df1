"""CPU tests of the oracle: pinned to the reference's own regression tests and fixtures,
cross-checked against an independent numpy/scipy/sympy restatement, and held to
mathematical known-answer tests (the reference ships no golden weights)."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rel_row_err

ALL6 = ("E", "Dx", "Dy", "Dxx", "Dyy", "Dxy")


def jgrid(pkg, nx, seed=1):
    return pkg.nodesets.jittered_grid(nx, seed=seed)[0]


def test_knn_grid_equals_brute_force(pkg, orc):
    X = jgrid(pkg, 40)
    rng = np.random.default_rng(0)
    Q = rng.uniform(-0.2, 1.2, (300, 2))  # includes queries outside the node box
    for k in (1, 7, 30, 64):
        a, da = orc.knn(X, Q, k)
        b, db = orc.knn(X, Q, k, brute=True)
        assert (a == b).all() and np.array_equal(da, db)
    a, _ = orc.knn(X, X, 30)
    assert (a[:, 0] == np.arange(len(X))).all()  # self first (sortres=true, distance 0)


def test_knn_ties_broken_by_index(orc):
    # an unjittered lattice has many exact ties in d^2
    g = (np.arange(12) + 0.5) / 12
    X = np.stack(np.meshgrid(g, g), -1).reshape(-1, 2)
    a, da = orc.knn(X, X, 13)
    b, db = orc.knn(X, X, 13, brute=True)
    assert (a == b).all()
    for i in range(len(X)):
        keys = list(zip(da[i], a[i]))
        assert keys == sorted(keys)


def test_knn_boundary_mask_brute(pkg, orc):
    d = pkg.nodesets.rectangle_with_ghosts(total=3000, seed=2)
    X, cls = d["X"], d["node_class"]
    a, _ = orc.knn(X, X, 20, cls_x=cls, cls_q=cls)
    b, _ = orc.knn(X, X, 20, cls_x=cls, cls_q=cls, brute=True)
    assert (a == b).all()
    for bb in range(1, 5):
        c = cls[a[cls == bb]]
        assert ((c >= 0) | (c == -bb)).all()
        c = cls[a[cls == -bb]]
        assert ((c >= 0) | (c == -bb)).all()


def test_oracle_matches_numpy_mirror(pkg, orc):
    from oracle import numpy_mirror as nm

    pytest.importorskip("sympy")
    X = jgrid(pkg, 24)
    ops = ALL6 + ("Lap",)
    cols, W = nm.generate(X, X, 3, 15, 2, ops)
    r = orc.generate(X, X, 3, 15, 2, ops)
    assert (cols == r["cols"]).all()
    for q in range(len(ops)):
        assert rel_row_err(W[q], r["W"][q]) < 1e-10, ops[q]
    Y = X[::5] + 3e-3
    cols, W = nm.generate(X, Y, 5, 30, 3, ("Dxk", "Dyk", "HV"), k_deriv=4)
    r = orc.generate(X, Y, 5, 30, 3, ("Dxk", "Dyk", "HV"), k_deriv=4)
    assert (cols == r["cols"]).all()
    for q in range(3):
        assert rel_row_err(W[q], r["W"][q]) < 1e-9


def test_phi_closed_forms_match_symbolic(orc):
    sympy = pytest.importorskip("sympy")
    x, y = sympy.symbols("x y", real=True)
    pts = [(0.3, -0.7), (-1.1, 0.2), (2.2e-16, 2.2e-16), (0.05, 1.3)]
    for p in (3, 5, 7):
        e = sympy.sqrt(x**2 + y**2) ** p
        for a, b in [(0, 0), (1, 0), (0, 1), (2, 0), (0, 2), (1, 1), (4, 0), (0, 4), (3, 1), (6, 0)]:
            d = sympy.diff(e, x, a) if a else e
            d = sympy.diff(d, y, b) if b else d
            f = sympy.lambdify((x, y), d, "mpmath")
            for px, py in pts:
                ref = float(f(sympy.Float(px, 50), sympy.Float(py, 50)))
                got = orc.phi(p, a, b, px, py)
                assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref)), (p, a, b, px, py, got, ref)


def test_poisson_regression_pin(orc, tominec):
    """test/poisson_test.jl:132 on the reference's own fixture: err < 0.0027."""
    from test_gpu_parity import poisson_error

    X = tominec["x_nodes"]
    Y = tominec["y_nodes"].copy()
    idx, _ = orc.knn(Y, X, 1)
    Y[idx[:, 0]] = X
    r = orc.generate(X, Y, 3, 20, 3, ALL6)
    M, N = len(Y), len(X)
    mats = []
    for q in range(6):
        cp, rv, nz = orc.to_csc(M, N, r["cols"], r["W"][q])
        mats.append(sp.csc_matrix((nz, rv - 1, cp - 1), shape=(M, N)))
    E, Dx, Dy, Dxx, Dyy, Dxy = mats
    err = poisson_error(X, Y, E, Dx, Dy, Dxx, Dyy, tominec, orc)
    assert err < 0.0027, err


def test_hyperviscosity_regression_pin(orc, tominec):
    """test/hyperviscosity_test.jl:32-33: Dxk(k=2) ~ Dxx, Dyk ~ Dyy with rtol sqrt(eps)."""
    X = tominec["x_nodes"]
    a = orc.generate(X, X, 5, 42, 5, ("Dxx", "Dyy"))
    b = orc.generate(X, X, 5, 42, 5, ("Dxk", "Dyk"), k_deriv=2)
    rtol = np.sqrt(np.finfo(float).eps)
    for q in range(2):
        assert np.linalg.norm(a["W"][q] - b["W"][q]) <= rtol * np.linalg.norm(a["W"][q])


@pytest.mark.parametrize("p,n,deg", [(3, 15, 2), (3, 30, 3), (5, 42, 5), (3, 60, 5)])
def test_polynomial_reproduction(pkg, orc, p, n, deg):
    """Every operator differentiates every monomial of degree <= deg exactly (to rounding)."""
    X = jgrid(pkg, 30, seed=3)
    Y = X[::7] + 1e-3
    ops = ALL6 + ("Lap",)
    r = orc.generate(X, Y, p, n, deg, ops)
    x, y = X[:, 0], X[:, 1]
    yx, yy = Y[:, 0], Y[:, 1]
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            f = x**a * y**b

            def d(i, j):
                if i > a or j > b:
                    return np.zeros_like(yx)
                c = np.prod(np.arange(a, a - i, -1)) * np.prod(np.arange(b, b - j, -1))
                return c * yx ** (a - i) * yy ** (b - j)

            exact = {"E": d(0, 0), "Dx": d(1, 0), "Dy": d(0, 1), "Dxx": d(2, 0), "Dyy": d(0, 2), "Dxy": d(1, 1),
                     "Lap": d(2, 0) + d(0, 2)}
            for q, o in enumerate(ops):
                got = (r["W"][q] * f[r["cols"]]).sum(1)
                scale = np.abs(r["W"][q]).sum(1) * np.abs(f[r["cols"]]).max(1) + 1.0
                assert (np.abs(got - exact[o]) <= 1e-10 * scale).all(), (o, a, b)


def test_collocated_identity_and_laplacian(pkg, orc):
    X = jgrid(pkg, 32, seed=4)
    r = orc.generate(X, X, 3, 20, 3, ("E", "Dxx", "Dyy", "Lap"))
    E = np.zeros((len(X), len(X)))
    E[np.repeat(np.arange(len(X)), 20), r["cols"].ravel()] = r["W"][0].ravel()
    assert np.abs(E - np.eye(len(X))).max() < 1e-10
    assert rel_row_err(r["W"][1] + r["W"][2], r["W"][3]) < 1e-9


@pytest.mark.parametrize("n,deg,ratio", [(15, 2, 1.4), (20, 3, 3.0)])
def test_laplacian_converges_under_refinement(pkg, orc, n, deg, ratio):
    """Manufactured f = sin(2 pi x) cos(3 pi y): the interior Lap error falls with h between
    32^2, 64^2 and 128^2 nodes -- first order for degree 2 (exact on quadratics), second
    order for degree 3 -- and Dx converges faster."""
    errs, errx = [], []
    for nx in (32, 64, 128):
        X, h, _ = pkg.nodesets.jittered_grid(nx, seed=1)
        f, fx, fy, lap = pkg.nodesets.manufactured(X)
        r = orc.generate(X, X, 3, n, deg, ("Lap", "Dx"))
        L = (r["W"][0] * f[r["cols"]]).sum(1)
        D = (r["W"][1] * f[r["cols"]]).sum(1)
        inner = (np.abs(X - 0.5) < 0.35).all(1)
        errs.append(np.abs(L - lap)[inner].max() / np.abs(lap).max())
        errx.append(np.abs(D - fx)[inner].max() / np.abs(fx).max())
    assert errs[0] > errs[1] * ratio and errs[1] > errs[2] * ratio, errs
    assert errx[0] > errx[1] * 2.5 and errx[1] > errx[2] * 2.5, errx


def test_csc_matches_scipy(pkg, orc):
    X = jgrid(pkg, 20)
    Y = X[::2] + 1e-3
    r = orc.generate(X, Y, 3, 12, 2, ("Dx",))
    cp, rv, nz = orc.to_csc(len(Y), len(X), r["cols"], r["W"][0])
    rows = np.repeat(np.arange(len(Y)), 12)
    A = sp.coo_matrix((r["W"][0].ravel(), (rows, r["cols"].ravel())), shape=(len(Y), len(X))).tocsc()
    A.sort_indices()
    assert np.array_equal(cp - 1, A.indptr) and np.array_equal(rv - 1, A.indices)
    assert np.array_equal(nz, A.data)
    x = np.random.default_rng(1).standard_normal(len(X))
    assert np.allclose(orc.spmv_csc(len(Y), cp, rv, nz, x), orc.spmv_rows(r["cols"], r["W"][0], x), atol=1e-12)


def test_singular_and_bad_input(pkg, orc):
    X = jgrid(pkg, 12)
    Xd = X.copy()
    Xd[3] = Xd[4]
    with pytest.raises(orc.OracleError) as e:
        orc.generate(Xd, Xd, 3, 10, 2, ("E",))
    assert e.value.code == orc.ORC_ESINGULAR
    with pytest.raises(orc.OracleError):
        orc.generate(X, X, 3, len(X) + 1, 2, ("E",))


@pytest.mark.parametrize("reverse", [False, True])
def test_process_mesh_oracle_against_numpy(orc, reverse):
    """processmesh after the file reads (src/processmesh.jl:1-192): the oracle's centroids,
    midpoints, normals and tangents equal a numpy restatement bit for bit; the nearest
    centroids are checked by brute force; normals end up pointing out of the square whichever
    way the boundary is listed; ghost nodes sit one offset outside the midpoints."""
    from conftest import rect_tri_mesh

    V, tri, markers = rect_tri_mesh(12, 9, seed=3, reverse=reverse)
    bc = np.concatenate(markers)
    Y, nrm, tng, off = orc.process_mesh(V, tri, bc)
    ntri, nbc = len(tri), len(bc)
    a, b, c = V[tri[:, 0] - 1], V[tri[:, 1] - 1], V[tri[:, 2] - 1]
    C = (a + b + c) / 3.0
    assert np.array_equal(Y[:ntri], C)
    p, q = V[bc[:, 0] - 1], V[bc[:, 1] - 1]
    M = (p + q) / 2.0
    assert np.array_equal(Y[ntri:ntri + nbc], M)
    d = q - p
    ln = np.sqrt(d[:, 1] * d[:, 1] + d[:, 0] * d[:, 0])
    n0 = np.stack([-d[:, 1] / ln, d[:, 0] / ln], axis=1)
    t0 = np.stack([d[:, 0] / ln, d[:, 1] / ln], axis=1)
    d2 = ((M[:, None, :] - C[None, :, :]) ** 2).sum(-1)
    nn = d2.argmin(1)
    sg = np.sign(np.dot(M[0] - C[nn[0]], n0[0]))
    assert np.array_equal(nrm, sg * n0) and np.array_equal(tng, sg * t0)
    assert off == pytest.approx(np.sqrt(d2[np.arange(nbc), nn]).mean(), rel=1e-14)
    assert np.allclose(Y[ntri + nbc:], M + nrm * off, rtol=0, atol=1e-15)
    # outward: bottom (0, -1), right (1, 0), top (0, 1), left (-1, 0)
    k = np.cumsum([0] + [len(m) for m in markers])
    for (i, want) in enumerate([(0, -1), (1, 0), (0, 1), (-1, 0)]):
        assert np.allclose(nrm[k[i]:k[i + 1]].mean(0), want, atol=1e-12)
    assert (Y[ntri + nbc:, 0] < -0.5 * off + 1e-12).sum() == len(markers[3])  # left ghosts outside
