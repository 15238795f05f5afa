"""The oracle's discrete RK4 adjoint against central finite differences of the
oracle's own RK4 forward (h = 1e-6 relative), on a small two-stage run shaped
like the flocculation adjoint workload: Brownian + shear aggregation with the
shear rate switching mid-run, power-law selection, power-law daughter, loss
L = sum x^(2/3) N(T). CPU only."""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle

pytestmark = pytest.mark.filterwarnings("ignore")


def setup(n=40, steps=6):
    x = pg.grids.geometric_pow2(n, 1e-21, 4.0)
    N0 = pg.grids.lognormal_ic(x, 10, 1.0, 1e14)
    t_q, bw_q = pg.quadrature.power_law(2.0, 4)
    v_ref = float(x[n // 2])
    agg = np.array([[5, 0.0, 6.73e-18, 4 * 100 / 3], [5, 0.0, 6.73e-18, 4 * 20 / 3]])
    brk = np.array([[2, 5e-4, v_ref, 1.0, 0.0], [2, 5e-4, v_ref, 1.0, 0.0]])
    step_set = np.array([0] * (steps // 2) + [1] * (steps - steps // 2))
    return x, N0, t_q, bw_q, agg, brk, step_set


def forward(N0, x, dt, step_set, agg, brk, t_q, bw_q):
    N = N0.copy()
    for s in step_set:
        a, b = agg[s], brk[s]
        N = pyoracle.rk4_step(N, x, dt, agg=dict(kernel=int(a[0]), beta0=a[1], beta_br=a[2],
                                                 beta_sh=a[3]),
                              brk=dict(t_q=t_q, bw_q=bw_q, selection=int(b[0]), S0=b[1],
                                       v_ref=b[2], alpha=b[3], v_min=b[4]))
    return N


def test_rk4_adjoint_matches_finite_differences():
    x, N0, t_q, bw_q, agg, brk, step_set = setup()
    dt = 0.5
    w = x ** (2.0 / 3.0)
    NT, gN0, ga, gb = pyoracle.rk4_adjoint(N0, x, dt, len(step_set), w, agg, brk, step_set,
                                           t_q, bw_q)
    ref_NT = forward(N0, x, dt, step_set, agg, brk, t_q, bw_q)
    np.testing.assert_allclose(NT, ref_NT, rtol=1e-14, atol=1e-300)

    def L(N0_=N0, agg_=agg, brk_=brk):
        return float(w @ forward(N0_, x, dt, step_set, agg_, brk_, t_q, bw_q))

    for m in (0, 5, 10, 14, 25):
        h = 1e-6 * N0[m]
        Np, Nm = N0.copy(), N0.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (L(Np) - L(Nm)) / (2 * h)
        assert abs(fd - gN0[m]) <= 1e-6 * abs(gN0[m]) + 1e-12 * abs(L()) / h, (m, fd, gN0[m])
    # coefficients, per parameter set: beta_br (col 2 of agg), beta_sh (3), S0 (brk col 1), alpha (3)
    for table, col, grad, gcol in ((agg, 2, ga, 1), (agg, 3, ga, 2), (brk, 1, gb, 0), (brk, 3, gb, 2)):
        for m in range(2):
            base = table[m, col]
            h = 1e-6 * base
            tp, tm = table.copy(), table.copy()
            tp[m, col] += h
            tm[m, col] -= h
            if table is agg:
                fd = (L(agg_=tp) - L(agg_=tm)) / (2 * h)
            else:
                fd = (L(brk_=tp) - L(brk_=tm)) / (2 * h)
            g = grad[m, gcol]
            assert abs(fd - g) <= 2e-6 * abs(g) + 1e-12 * abs(L()) / h, (col, m, fd, g)


def test_rk4_adjoint_zero_steps_is_identity():
    x, N0, t_q, bw_q, agg, brk, _ = setup(n=12)
    lam = np.linspace(1.0, 2.0, len(x))
    NT, gN0, ga, gb = pyoracle.rk4_adjoint(N0, x, 0.5, 0, lam, agg, brk, None, t_q, bw_q)
    assert np.array_equal(NT, N0) and np.array_equal(gN0, lam)
    assert not ga.any() and not gb.any()
