"""The oracle's vector-Jacobian products agree with central finite differences
of the oracle's own forward RHS (CPU). This pins the adjoint arithmetic the
GPU VJP kernels are later compared with.

L(N, p) = lambda . rhs(N, p) is quadratic in N for aggregation (so central
differences are exact up to rounding) and linear in N for breakage; in the
parameters it is linear (beta) or smooth (S0, v_ref, alpha). Step h = 1e-6
relative; the bound allows the differencing noise."""
import math

import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle

AGG = [(0, 1e-15, 0.0, 0.0), (1, 1e-3, 0.0, 0.0), (2, 1e12, 0.0, 0.0), (3, 0.0, 6.73e-18, 0.0),
       (4, 0.0, 0.0, 66.67), (5, 0.0, 6.73e-18, 66.67)]


def _setup(n=40, seed=0):
    rng = np.random.default_rng(seed)
    x = pg.grids.geometric_pow2(n, 1e-21, 6.0)
    N = rng.lognormal(20.0, 1.0, n)
    lam = rng.normal(size=n)
    return x, N, lam


def _L_agg(N, x, lam, k, b0, bbr, bsh):
    r, _, _ = pyoracle.aggregation_rhs(N, x, k, b0, bbr, bsh, math.log(x[0]),
                                       1.0 / math.log(x[1] / x[0]), exact_bracket=True)
    return float(np.dot(lam, r))


@pytest.mark.parametrize("k,b0,bbr,bsh", AGG)
def test_aggregation_vjp_matches_finite_differences(k, b0, bbr, bsh):
    x, N, lam = _setup(seed=k)
    gN, gp, code = pyoracle.aggregation_rhs_vjp(N, x, lam, k, b0, bbr, bsh,
                                                math.log(x[0]), 1.0 / math.log(x[1] / x[0]))
    assert code == 0
    scale = abs(_L_agg(N, x, np.abs(lam), k, b0, bbr, bsh)) or 1.0
    for m in range(0, len(x), 7):
        h = 1e-6 * N[m]
        Np, Nm = N.copy(), N.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (_L_agg(Np, x, lam, k, b0, bbr, bsh) - _L_agg(Nm, x, lam, k, b0, bbr, bsh)) / (2 * h)
        assert abs(fd - gN[m]) <= 1e-7 * scale / N[m] + 1e-9 * abs(gN[m]), (m, fd, gN[m])
    for idx, (name, val) in enumerate((("beta0", b0), ("beta_br", bbr), ("beta_sh", bsh))):
        if val == 0.0:
            continue
        h = 1e-6 * val
        args = [b0, bbr, bsh]
        ap, am = list(args), list(args)
        ap[idx] += h
        am[idx] -= h
        fd = (_L_agg(N, x, lam, k, *ap) - _L_agg(N, x, lam, k, *am)) / (2 * h)
        assert abs(fd - gp[idx]) <= 1e-7 * scale / val, (name, fd, gp[idx])


SEL = [(0, 1e-3, 1.0, 1.0, 0.0), (1, 1e-3, "mid", 1.0, 0.0), (2, 5e-4, "mid", 1.5, 0.0),
       (3, 1e-3, 1.0, 1.0, "mid")]


@pytest.mark.parametrize("sel,S0,vref,alpha,vmin", SEL)
@pytest.mark.parametrize("daughter", ["uniform", "powerlaw", "erosion"])
def test_breakage_vjp_matches_finite_differences(sel, S0, vref, alpha, vmin, daughter):
    x, N, lam = _setup(seed=10 + sel)
    mid = float(x[len(x) // 2])
    vref = mid if vref == "mid" else vref
    vmin = mid if vmin == "mid" else vmin
    t_q, bw_q = {"uniform": pg.quadrature.uniform(6), "powerlaw": pg.quadrature.power_law(2.0, 3),
                 "erosion": pg.quadrature.erosion(0.05)}[daughter]

    def L(N_, S0_=S0, vref_=vref, alpha_=alpha):
        r, _, _ = pyoracle.breakage_rhs(N_, x, t_q, bw_q, sel, S0_, vref_, alpha_, vmin)
        return float(np.dot(lam, r))

    gN, gp, code = pyoracle.breakage_rhs_vjp(N, x, t_q, bw_q, lam, sel, S0, vref, alpha, vmin)
    assert code == 0
    for m in range(0, len(x), 5):
        h = 1e-6 * N[m]
        Np, Nm = N.copy(), N.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (L(Np) - L(Nm)) / (2 * h)
        assert abs(fd - gN[m]) <= 1e-7 * (abs(gN[m]) + S0), (m, fd, gN[m])
    scale = abs(float(np.dot(np.abs(lam), np.abs(pyoracle.breakage_rhs(N, x, t_q, bw_q, sel, S0, vref,
                                                                          alpha, vmin)[0]))))
    for idx, kw in ((0, "S0_"), (1, "vref_"), (2, "alpha_")):
        base = {"S0_": S0, "vref_": vref, "alpha_": alpha}[kw]
        h = 1e-6 * base
        fd = (L(N, **{kw: base + h}) - L(N, **{kw: base - h})) / (2 * h)
        assert abs(fd - gp[idx]) <= 1e-6 * scale / base, (kw, fd, gp[idx])
