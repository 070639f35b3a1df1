"""RK4 time stepping (rbffd_rk4_*) on the paths the stage-form test in test_gpu_parity.py does
not reach: the tiled FP32 stage kernel on ragged rows (per-node stencil sizes, so tiles mix row
lengths and pad them) and on every field count it takes, against an FP64 numpy RK4 of the same
operator (the time loop of examples/adv_diff_test.jl:144-199 with held boundary rows).

The library evaluates classic RK4 for this constant linear operator in Horner form and the
FP32 operator in difference form; both equal the stage form in exact arithmetic, so the numpy
reference is the plain stage form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rk4_numpy(L, fixed, U0, dt, nsteps):
    def f(u):
        v = L @ u
        v[fixed] = 0.0
        return v

    u = U0.copy()
    for _ in range(nsteps):
        k1 = f(u)
        k2 = f(u + 0.5 * dt * k1)
        k3 = f(u + 0.5 * dt * k2)
        k4 = f(u + dt * k3)
        u = u + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    return u


@pytest.mark.parametrize("F", [4, 8, 16, 32, 64, 128])
def test_rk4_ragged_rows_tiled(pkg, gpu, F):
    """Per-node (k, degree) classes (20..60 nodes per row): rows of one tile have different
    lengths.  FP32 (tiled kernel) within 2e-5 and FP64 within 1e-10 of the FP64 reference."""
    import torch

    d = pkg.nodesets.rectangle_with_ghosts(total=5000, seed=31, main_fraction=0.5)
    X, cls, nn, dd = d["X"], d["node_class"], d["n"], d["deg"]
    ops = ("Dx", "Dy", "Lap")
    coef = [-1.0, -0.5, 2e-3]
    with pkg.OperatorSet(X, None, 3, 0, 0, ops=ops, node_class=cls, n_per_node=nn, deg_per_node=dd) as s:
        L = sum(c * s.csr(o) for c, o in zip(coef, ops))
        fixed = cls != 0
        h = 1.0 / np.sqrt(len(X) / 2.0)
        dt, nsteps = 0.05 * h, 5
        U0 = np.random.default_rng(7).standard_normal((len(X), F))
        ref = rk4_numpy(L, fixed, U0, dt, nsteps)
        for dtype, tol in (("f32", 2e-5), ("f64", 1e-10)):
            td = torch.float32 if dtype == "f32" else torch.float64
            with pkg.RK4Stepper([s], coef, F, dtype, fixed_rows=fixed) as st:
                ud = torch.tensor(U0, dtype=td, device="cuda")
                st.run(ud, dt, nsteps)
                got = ud.double().cpu().numpy()
            err = np.abs(got - ref).max() / np.abs(ref).max()
            assert err <= tol, (dtype, F, err)
            held = U0[fixed].astype(np.float32 if dtype == "f32" else np.float64).astype(np.float64)
            assert np.array_equal(got[fixed], held)


def test_rk4_odd_step_counts_and_restart(pkg, orc, gpu):
    """1 step, 2 steps (one replay of the two-step graph) and 3 steps from the same start, FP32
    tiled: each matches the reference, so the single-step tail and graph replays agree."""
    import scipy.sparse as sp
    import torch

    X, h, _ = pkg.nodesets.jittered_grid(40, seed=33)
    N, n = len(X), 30
    ops = ("Dx", "Dy", "Lap")
    coef = [-1.0, -0.5, 1e-2]
    ref_ops = orc.generate(X, X, 3, n, 3, ops)
    rows = np.repeat(np.arange(N), n)
    L = sum(c * sp.csr_matrix((ref_ops["W"][q].ravel(), (rows, ref_ops["cols"].ravel())), shape=(N, N))
            for q, c in enumerate(coef))
    fixed = ((X < 1.5 * h) | (X > 1 - 1.5 * h)).any(1)
    F = 64
    U0 = np.random.default_rng(9).standard_normal((N, F))
    dt = 0.1 * h
    with pkg.OperatorSet(X, None, 3, n, 3, ops=ops) as s, pkg.RK4Stepper([s], coef, F, "f32", fixed_rows=fixed) as st:
        for nsteps in (1, 2, 3):
            ud = torch.tensor(U0, dtype=torch.float32, device="cuda")
            st.run(ud, dt, nsteps)
            ref = rk4_numpy(L, fixed, U0, dt, nsteps)
            err = np.abs(ud.double().cpu().numpy() - ref).max() / np.abs(ref).max()
            assert err <= 2e-5, (nsteps, err)
