"""CPU check of the closed-form right-hand sides that the register Schur kernel uses instead
of its term table (csrc/schur.cuh, build_rhs_schur): the identities are verified
symbolically, and numerically against the oracle's derivatives of the basis
(oracle/rbffd_oracle.c orc_phi, itself checked against sympy in test_oracle.py).

  r^3:  d/dx = 3 x r,  d2/dx2 = 3 r + 3 x^2 / r,  d2/dxdy = 3 x y / r,
        sx^2 d2/dx2 + sy^2 d2/dy2 = (3 (2 sx^2 + sy^2) x^2 + 3 (sx^2 + 2 sy^2) y^2) / r
  r^5:  d4/dx4 = 15 r (3 + 6 u - u^2),  u = x^2 / r^2
  polynomial rows at the centre: d^(a+b)/dx^a dy^b of x^a y^b is a! b!, every other
  monomial of the basis gives 0.
"""
import math

import numpy as np
import pytest


def test_closed_forms_symbolic():
    sp = pytest.importorskip("sympy")
    x, y, sx, sy = sp.symbols("x y s_x s_y", positive=True)
    r = sp.sqrt(x**2 + y**2)
    r3, r5 = r**3, r**5
    assert sp.simplify(sp.diff(r3, x) - 3 * x * r) == 0
    assert sp.simplify(sp.diff(r3, x, 2) - (3 * r + 3 * x**2 / r)) == 0
    assert sp.simplify(sp.diff(r3, x, y) - 3 * x * y / r) == 0
    lap = sx**2 * sp.diff(r3, x, 2) + sy**2 * sp.diff(r3, y, 2)
    closed = (3 * (2 * sx**2 + sy**2) * x**2 + 3 * (sx**2 + 2 * sy**2) * y**2) / r
    assert sp.simplify(lap - closed) == 0
    u = x**2 / r**2
    assert sp.simplify(sp.diff(r5, x, 4) - 15 * r * (3 + 6 * u - u**2)) == 0


def test_closed_forms_match_oracle_basis_derivatives(orc):
    rng = np.random.default_rng(12)
    P = rng.uniform(-1.0, 1.0, (200, 2))
    sx, sy = 1.7, 0.6
    for px, py in P:
        rr = math.hypot(px, py)
        assert orc.phi(3, 1, 0, px, py) == pytest.approx(3 * px * rr, rel=1e-13, abs=1e-15)
        assert orc.phi(3, 2, 0, px, py) == pytest.approx(3 * rr + 3 * px * px / rr, rel=1e-13)
        assert orc.phi(3, 1, 1, px, py) == pytest.approx(3 * px * py / rr, rel=1e-13, abs=1e-15)
        lap = sx**2 * orc.phi(3, 2, 0, px, py) + sy**2 * orc.phi(3, 0, 2, px, py)
        closed = (3 * (2 * sx**2 + sy**2) * px**2 + 3 * (sx**2 + 2 * sy**2) * py**2) / rr
        assert lap == pytest.approx(closed, rel=1e-13)
        u = px * px / (rr * rr)
        assert orc.phi(5, 4, 0, px, py) == pytest.approx(15 * rr * (3 + 6 * u - u * u), rel=1e-12)


def test_polynomial_rows_at_the_centre():
    sp = pytest.importorskip("sympy")
    x, y = sp.symbols("x y")
    for deg in range(6):
        mons = [x ** (t - b) * y**b for t in range(deg + 1) for b in range(t + 1)]  # index t(t+1)/2 + b
        for a in range(5):
            for b in range(5 - a):
                vals = [sp.diff(mon, x, a, y, b).subs({x: 0, y: 0}) if (a or b) else mon.subs({x: 0, y: 0})
                        for mon in mons]
                t = a + b
                want = [0] * len(mons)
                if t <= deg:
                    want[t * (t + 1) // 2 + b] = math.factorial(a) * math.factorial(b)
                assert vals == want, (deg, a, b)
