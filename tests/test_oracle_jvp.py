"""The oracle's Jacobian-vector products (oracle/pbe_oracle.cpp) and its dense
ROS2 step, pinned without a GPU:

* aggregation: the RHS is quadratic in N, so the central difference
  (R(N + s v) - R(N - s v)) / 2s equals J(N) v up to round-off for any s;
* breakage: linear in N where the guard passes, so R(N + s v) - R(N) = s J v
  when N and N + s v pass the guard in the same bins, and the bins that fail
  the guard contribute nothing;
* ROS2: second order (halving dt divides the error against a fine RK4
  solution by ~4) and exact for a linear decay (breakage only, one bin).
"""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle as po

KERNELS = [(0, 1e-15, 0.0, 0.0), (1, 1e-3, 0.0, 0.0), (2, 1e12, 0.0, 0.0),
           (3, 0.0, 6.73e-18, 0.0), (4, 0.0, 0.0, 66.67), (5, 0.0, 6.73e-18, 66.67)]


def _case(rng, n, q):
    x = 1e-18 * 2.0 ** (np.arange(n) / q)
    N = rng.lognormal(20.0, 2.0, n)
    N[rng.random(n) < 0.2] = 0.0
    return x, N


@pytest.mark.parametrize("kernel,b0,bbr,bsh", KERNELS, ids=[str(k[0]) for k in KERNELS])
@pytest.mark.parametrize("q", [1, 4, 32])
def test_aggregation_jvp_equals_central_difference(kernel, b0, bbr, bsh, q):
    rng = np.random.default_rng(10 * kernel + q)
    for n in (1, 2, 17, 60):
        x, N = _case(rng, n, q)
        v = rng.normal(size=n) * max(N.max(), 1.0)
        jv, scale, code = po.aggregation_rhs_jvp(N, v, x, kernel, b0, bbr, bsh)
        assert code == 0
        s = 1e-2
        fp = po.aggregation_rhs(N + s * v, x, kernel, b0, bbr, bsh, exact_bracket=True)[0]
        fm = po.aggregation_rhs(N - s * v, x, kernel, b0, bbr, bsh, exact_bracket=True)[0]
        fd = (fp - fm) / (2.0 * s)
        tol = 1e-12 * (np.abs(fp).max() + np.abs(fm).max()) / s + 1e-300
        assert np.max(np.abs(jv - fd)) <= tol, (n, q)


@pytest.mark.parametrize("sel", [0, 1, 2, 3])
def test_breakage_jvp_is_the_guarded_linear_part(sel):
    rng = np.random.default_rng(50 + sel)
    t_q, bw_q = pg.quadrature.uniform(4)
    n = 40
    x = 1e-18 * 2.0 ** (np.arange(n) / 8)
    N = rng.lognormal(20.0, 2.0, n)
    N[::7] = 0.0                       # fails the guard
    N[3] = -5.0                        # fails the guard
    v = rng.normal(size=n) * 1e8
    prm = dict(S0=1e-3, v_ref=float(x[n // 2]), alpha=1.3, v_min=float(x[n // 3]))
    jv, _, code = po.breakage_rhs_jvp(N, v, x, t_q, bw_q, sel, **prm)
    assert code == 0
    # the same with v zeroed where N fails the guard: identical
    v2 = np.where(N > 2.2e-308, v, 0.0)
    jv2 = po.breakage_rhs_jvp(N, v2, x, t_q, bw_q, sel, **prm)[0]
    np.testing.assert_array_equal(jv, jv2)
    # linearity on the bins that pass the guard (N + s v keeps its sign there)
    live = N > 2.2e-308
    s = 1e-3 * np.min(N[live] / np.maximum(np.abs(v[live]), 1e-300))
    vv = np.where(live, v, 0.0)
    f0 = po.breakage_rhs(N, x, t_q, bw_q, sel, **prm)[0]
    f1 = po.breakage_rhs(N + s * vv, x, t_q, bw_q, sel, **prm)[0]
    scale = np.abs(f0).max() + np.abs(f1).max()
    np.testing.assert_allclose((f1 - f0) / s, jv, rtol=0, atol=1e-9 * scale / s)


def test_ros2_oracle_is_second_order():
    n = 24
    x = 1e-18 * 2.0 ** (np.arange(n) / 2)
    N0 = pg.grids.lognormal_ic(x, 6, 1.0, 1e14)
    agg = dict(kernel=5, beta_br=6.73e-18, beta_sh=66.67)
    t_q, bw_q = pg.quadrature.uniform(4)
    brk = dict(t_q=t_q, bw_q=bw_q, selection=2, S0=1e-2, v_ref=float(x[n // 2]), alpha=1.0)
    T = 8.0
    ref = N0.copy()
    for _ in range(800):
        ref = po.rk4_step(ref, x, T / 800, agg, brk)
    errs = []
    for steps in (8, 16, 32):
        N = N0.copy()
        for _ in range(steps):
            N = po.ros2_step(N, x, T / steps, agg, brk)
        errs.append(np.abs(N - ref).max() / np.abs(ref).max())
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 3.0 < r1 < 5.5 and 3.0 < r2 < 5.5, errs


def test_ros2_oracle_is_l_stable_on_a_stiff_decay():
    """One bin with breakage only, every fragment clipped back into it with
    weight 1/2: dN/dt = S (1/2 - 1) N. ROS2's stability function at z = lam dt
    is R(z) = (1 + (1 - 2 g) z + (1/2 - 2 g + g^2) z^2) / (1 - g z)^2, which
    tends to 0 as z -> -inf (L-stable)."""
    x = np.array([1e-18])
    brk = dict(t_q=np.array([0.5]), bw_q=np.array([0.5]), selection=0, S0=2e3)
    N = np.array([1e10])
    g = 1.0 + 1.0 / np.sqrt(2.0)
    for dt in (1e-6, 1e-3, 1.0, 1e3):
        z = -1e3 * dt
        R = (1 + (1 - 2 * g) * z + (0.5 - 2 * g + g * g) * z * z) / (1 - g * z) ** 2
        got = po.ros2_step(N, x, dt, None, brk)[0]
        assert abs(got - R * N[0]) <= 1e-12 * N[0], (dt, got, R * N[0])
    assert abs(R) < 1e-3
