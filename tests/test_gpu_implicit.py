"""Jacobian-vector products and the linearly implicit ROS2 integrator of the
batched plan (pbe_batch_jvp, pbe_batch_ros2).

* JVP: every cell of mixed batches (geometric / generic grids, n from 1 up,
  every aggregation kernel, with and without breakage, N with zeros and a
  negative bin) against the oracle's J(N) v: |gpu - oracle| <= 1e-12 scale.
* ROS2: with a Krylov dimension >= n the GMRES solve is exact (up to
  round-off), so the steps match the oracle's dense-Jacobian ROS2 cell by
  cell; with a small dimension on a stiff case (where explicit RK4 blows up)
  they follow the dense-solve ROS2 closely and converge at second order to a
  fine RK4 reference. Repeated runs are bitwise identical."""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import assert_close, t
from test_gpu_batch import DAUGHTER, mixed_batch

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    return torch


def oracle_jvp(Nc, vc, x, kernel, selection, prm, t_q, bw_q):
    out = np.zeros(len(x))
    sc = np.zeros(len(x))
    if kernel >= 0:
        r, s, code = pyoracle.aggregation_rhs_jvp(Nc, vc, x, kernel, prm[0], prm[1], prm[2])
        assert code == 0
        out += r
        sc += s
    if selection >= 0:
        r, s, code = pyoracle.breakage_rhs_jvp(Nc, vc, x, t_q, bw_q, selection, prm[3], prm[4],
                                               prm[5], prm[6])
        assert code == 0
        out += r
        sc += s
    return out, sc


def _dicts(kernel, selection, prm, t_q, bw_q):
    agg = None if kernel < 0 else dict(kernel=kernel, beta0=prm[0], beta_br=prm[1], beta_sh=prm[2])
    brk = None if selection < 0 else dict(t_q=t_q, bw_q=bw_q, selection=selection, S0=prm[3],
                                          v_ref=prm[4], alpha=prm[5], v_min=prm[6])
    return agg, brk


@pytest.mark.parametrize("selection", [-1, 2])
@pytest.mark.parametrize("kernel", [-1, 0, 1, 2, 3, 4, 5])
def test_batch_jvp_matches_oracle_per_cell(kernel, selection):
    if kernel < 0 and selection < 0:
        pytest.skip("a plan needs aggregation or breakage")
    torch = _torch()
    rng = np.random.default_rng(300 + 7 * kernel + selection)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, kernel, selection, n_cells=30,
                                                      n_max=200)
    N[5][0] = -3.0 * abs(N[5]).max()              # a negative bin fails the breakage guard
    V = [rng.normal(size=len(Nc)) * max(np.abs(Nc).max(), 1.0) for Nc in N]
    t_q, bw_q = DAUGHTER
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel, selection, t_q, bw_q) as plan:
        dN, dv = t(np.concatenate(N)), t(np.concatenate(V))
        out = t(np.full(plan.total, 7.0))           # overwritten
        assert plan.jvp(dN, dv, out, t(params)) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for c in range(len(cell_n)):
            x = grids[cell_grid[c]][:cell_n[c]]
            ref, sc = oracle_jvp(N[c], V[c], x, kernel, selection, params[c], t_q, bw_q)
            o = plan.offsets[c]
            assert_close(got[o:o + cell_n[c]], ref, sc, "jvp k=%d sel=%d cell %d (n=%d)"
                         % (kernel, selection, c, cell_n[c]))


@pytest.mark.parametrize("kernel,selection", [(5, 2), (3, -1), (1, 0), (-1, 3)])
def test_ros2_full_krylov_matches_dense_oracle(kernel, selection):
    """krylov_dim >= n: GMRES reaches the exact solution, so each step equals
    the oracle's dense-Jacobian ROS2 step."""
    torch = _torch()
    rng = np.random.default_rng(900 + kernel + selection)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, kernel, selection, n_cells=12,
                                                      n_max=40)
    N = [np.abs(Nc) for Nc in N]
    t_q, bw_q = DAUGHTER
    dt, steps = 0.5, 3
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel, selection, t_q, bw_q) as plan:
        dN = t(np.concatenate(N))
        resid = t(np.zeros(len(cell_n)))
        code = plan.ros2(dN, t(params), dt, steps, krylov_dim=48, resid=resid)
        assert code == 0, pg.error_string(code)
        torch.cuda.synchronize()
        got = dN.cpu().numpy()
        rs = resid.cpu().numpy()
    assert np.all(rs < 1e-10), rs
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        agg, brk = _dicts(kernel, selection, params[c], t_q, bw_q)
        ref = N[c].copy()
        for _ in range(steps):
            ref = pyoracle.ros2_step(ref, x, dt, agg, brk)
        o = plan.offsets[c]
        sc = np.abs(ref).max() + np.abs(N[c]).max() + 1e-300
        err = np.abs(got[o:o + cell_n[c]] - ref).max() / sc
        assert err < 1e-9, (c, cell_n[c], err)


def test_ros2_stiff_steps_with_small_krylov_and_determinism():
    """Fast breakage (S0 dt up to ~1e4 in the largest bins) with Brownian+shear
    aggregation: explicit RK4 at dt = 1 blows up, ROS2 with GMRES(16) stays on
    the oracle's dense-solve ROS2 (relative 1e-5: the Krylov solve is not
    exact; the method's own error at dt = 1 is ~0.12) and converges to a fine
    RK4 solution at second order."""
    torch = _torch()
    n = 64
    x = 1e-18 * 2.0 ** (np.arange(n) / 4)
    N0 = pg.grids.lognormal_ic(x, 20, 1.0, 1e12)
    t_q, bw_q = pg.quadrature.uniform(4)
    S0, T = 50.0, 4.0
    prm = pg.batch.cell_params(2, beta_br=6.73e-18, beta_sh=66.67, S0=S0, v_ref=float(x[n // 2]),
                               alpha=1.0)
    agg = dict(kernel=5, beta_br=6.73e-18, beta_sh=66.67)
    brk = dict(t_q=t_q, bw_q=bw_q, selection=1, S0=S0, v_ref=float(x[n // 2]), alpha=1.0)
    fine = N0.copy()
    for _ in range(4000):
        fine = pyoracle.rk4_step(fine, x, T / 4000, agg, brk)
    errs = []
    with pg.BatchPlan([x], [n, n], [0, 0], 5, 1, t_q, bw_q) as plan:
        for steps in (4, 8):
            dt = T / steps
            outs = []
            for _ in range(2):
                dN = t(np.concatenate([N0, N0]))
                assert plan.ros2(dN, t(prm), dt, steps, krylov_dim=16) == 0
                torch.cuda.synchronize()
                outs.append(dN.cpu().numpy())
            a = outs[0]
            np.testing.assert_array_equal(a.view(np.int64), outs[1].view(np.int64))
            np.testing.assert_array_equal(a[:n].view(np.int64), a[n:].view(np.int64))
            dense = N0.copy()
            for _ in range(steps):
                dense = pyoracle.ros2_step(dense, x, dt, agg, brk)
            assert np.abs(a[:n] - dense).max() <= 1e-5 * np.abs(dense).max()
            errs.append(np.abs(a[:n] - fine).max() / np.abs(fine).max())
        blow = t(np.concatenate([N0, N0]))
        assert plan.rk4(blow, t(prm), 1.0, 4) == 0
        torch.cuda.synchronize()
        rk = blow.cpu().numpy()
    assert errs[0] < 0.15 and errs[1] < errs[0] / 4, errs
    assert not np.all(np.abs(rk[:n] - fine) < 0.15 * np.abs(fine).max())   # explicit RK4 fails


def test_ros2_argument_errors():
    x = 1e-18 * 2.0 ** (np.arange(8) / 2)
    t_q, bw_q = pg.quadrature.uniform(2)
    prm = pg.batch.cell_params(1, beta_br=6.73e-18, S0=1e-3)
    with pg.BatchPlan([x], [8], [0], 3, 0, t_q, bw_q) as plan:
        dN = t(np.ones(8))
        dp = t(prm)
        assert plan.ros2(dN, dp, 0.1, 1, krylov_dim=0) == pg.ERR_INVALID_VALUE
        assert plan.ros2(dN, dp, 0.1, 1, krylov_dim=65) == pg.ERR_INVALID_VALUE
        assert plan.ros2(dN, dp, -0.1, 1) == pg.ERR_INVALID_VALUE
        assert plan.ros2(dN, dp, 0.1, -1) == pg.ERR_INVALID_VALUE
        assert plan.ros2(dN, dp, 0.1, 0) == 0
        assert plan.jvp(0, dN, dN, dp) == pg.ERR_INVALID_DEVICE_POINTER


def test_ros2_adaptive_matches_dense_oracle_controller():
    """Exact solves (krylov_dim >= n): the per-cell step sequence (accepted and
    rejected steps) equals the oracle's controller run with dense solves."""
    torch = _torch()
    rng = np.random.default_rng(4242)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, 5, 2, n_cells=8, n_max=32,
                                                      kinds=("geo_fine", "geo_coarse"))
    N = [np.abs(Nc) for Nc in N]
    t_q, bw_q = DAUGHTER
    t_end, rtol, atol, dt0 = 4.0, 1e-4, 1e-6 * max(Nc.max() for Nc in N), 0.1
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        dN = t(np.concatenate(N))
        code, steps, rejects, att = plan.ros2_adaptive(dN, t(params), t_end, rtol, atol, dt0,
                                                       krylov_dim=40)
        assert code == 0, pg.error_string(code)
        torch.cuda.synchronize()
        got = dN.cpu().numpy()
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        agg, brk = _dicts(5, 2, params[c], t_q, bw_q)
        ref, st, rj, status = pyoracle.ros2_adaptive(N[c], x, t_end, rtol, atol, dt0, agg, brk)
        assert status == 1
        # the step sizes agree to round-off (GMRES vs dense LU): the counts may
        # differ by the last, shortest step
        assert abs(int(steps[c]) - st) <= 1 and rejects[c] == rj, (c, steps[c], rejects[c], st, rj)
        o = plan.offsets[c]
        sc = np.abs(ref).max() + 1e-300
        assert np.abs(got[o:o + cell_n[c]] - ref).max() <= 1e-8 * sc, c


def test_ros2_adaptive_on_a_persistently_stiff_cell():
    """Aggregation (G = 200 s^-1) against power-law breakage S ~ (x/v_ref)^2:
    the largest bins keep breaking at up to ~2.5e7 s^-1 while aggregation
    refills them, so an explicit method stays stability-limited throughout
    (RK45 does not reach t_end within 20000 attempts), while ROS2's steps are
    limited by accuracy only. Exact solves (krylov_dim >= n): the run follows
    the oracle's dense-solve controller."""
    torch = _torch()
    n = 40
    x = 1e-18 * 2.0 ** (np.arange(n) / 2)
    N0 = pg.grids.lognormal_ic(x, 8, 1.0, 1e14)
    t_q, bw_q = pg.quadrature.uniform(4)
    prm = pg.batch.cell_params(1, beta_br=6.73e-18, beta_sh=4 * 200 / 3, S0=1.0,
                               v_ref=float(x[14]), alpha=2.0)
    agg = dict(kernel=5, beta_br=6.73e-18, beta_sh=4 * 200 / 3)
    brk = dict(t_q=t_q, bw_q=bw_q, selection=2, S0=1.0, v_ref=float(x[14]), alpha=2.0)
    t_end, rtol, atol, dt0 = 20.0, 1e-3, 1e-6 * N0.max(), 1e-3
    ref, st, rj, status = pyoracle.ros2_adaptive(N0, x, t_end, rtol, atol, dt0, agg, brk)
    assert status == 1
    with pg.BatchPlan([x], [n], [0], 5, 2, t_q, bw_q) as plan:
        a, b = t(N0.copy()), t(N0.copy())
        code, steps, rejects, att = plan.ros2_adaptive(a, t(prm), t_end, rtol, atol, dt0,
                                                       krylov_dim=n)
        assert code == 0, pg.error_string(code)
        code_rk, s_rk, _, att_rk = plan.rk45(b, t(prm), t_end, rtol, atol, dt0,
                                             max_attempts=20000)
        torch.cuda.synchronize()
        A = a.cpu().numpy()
    assert code_rk == pg.ERR_NOT_READY and att_rk == 20000
    assert abs(int(steps[0]) - st) <= 1 and rejects[0] == rj, (steps, rejects, st, rj)
    assert att < 20000 // 4
    assert np.abs(A - ref).max() <= 1e-8 * np.abs(ref).max()


def test_krylov_tolerance_ends_solves_early_within_tolerance():
    """pbe_batch_set_krylov_tol: with tol = 1e-9 every solve stops once its
    relative least-squares residual is <= tol (the reported residuals are),
    the steps stay on the oracle's dense-solve ROS2 (relative 1e-6) but are
    not the full-dimension solves bit for bit (some solve stopped early); the
    adaptive controller with tol = 1e-9 takes the dense controller's steps.
    Tolerances outside [0, 1) are rejected."""
    torch = _torch()
    rng = np.random.default_rng(905)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, 5, 2, n_cells=12, n_max=40)
    N = [np.abs(Nc) for Nc in N]
    t_q, bw_q = DAUGHTER
    dt, steps = 0.5, 3
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        for bad in (-1e-3, 1.0, float("nan")):
            assert plan.set_krylov_tol(bad) == pg.ERR_INVALID_VALUE
        outs, rs = [], []
        for tol in (0.0, 1e-9):
            assert plan.set_krylov_tol(tol) == 0
            dN = t(np.concatenate(N))
            resid = t(np.zeros(len(cell_n)))
            code = plan.ros2(dN, t(params), dt, steps, krylov_dim=48, resid=resid)
            assert code == 0, pg.error_string(code)
            torch.cuda.synchronize()
            outs.append(dN.cpu().numpy())
            rs.append(resid.cpu().numpy())
        assert np.all(rs[1] <= 1e-9), rs[1]
        assert not np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64))
        for c in range(len(cell_n)):
            x = grids[cell_grid[c]][:cell_n[c]]
            agg, brk = _dicts(5, 2, params[c], t_q, bw_q)
            ref = N[c].copy()
            for _ in range(steps):
                ref = pyoracle.ros2_step(ref, x, dt, agg, brk)
            o = plan.offsets[c]
            sc = np.abs(ref).max() + np.abs(N[c]).max() + 1e-300
            assert np.abs(outs[1][o:o + cell_n[c]] - ref).max() / sc < 1e-6, c
        # adaptive
        t_end, rtol, dt0 = 4.0, 1e-4, 0.1
        atol = 1e-6 * max(Nc.max() for Nc in N)
        dN = t(np.concatenate(N))
        code, st, rj, att = plan.ros2_adaptive(dN, t(params), t_end, rtol, atol, dt0,
                                               krylov_dim=40)
        assert code == 0, pg.error_string(code)
        torch.cuda.synchronize()
        got = dN.cpu().numpy()
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        agg, brk = _dicts(5, 2, params[c], t_q, bw_q)
        ref, s_o, r_o, status = pyoracle.ros2_adaptive(N[c], x, t_end, rtol, atol, dt0, agg, brk)
        assert status == 1
        assert abs(int(st[c]) - s_o) <= 1 and abs(int(rj[c]) - r_o) <= 1, (c, st[c], rj[c], s_o, r_o)
        o = plan.offsets[c]
        assert np.abs(got[o:o + cell_n[c]] - ref).max() <= 1e-6 * (np.abs(ref).max() + 1e-300), c


def test_krylov_restarts_reach_the_tolerance_with_a_small_dimension():
    """Restarted GMRES: a ROS2 step (dt = 1 s, Brownian+shear + linear
    breakage, n = 64) solved with a Krylov dimension too small for one cycle
    (S0 = 1 s^-1 with m = 4: relative residual ~4e-4; S0 = 50 s^-1 with
    m = 12: ~4e-6) reaches tol = 1e-12 within 10 restarts, and the step then
    equals the oracle's dense-solve ROS2 step (relative 1e-11 and 1e-8). (With
    m <= 8 at S0 = 50 restarted GMRES stagnates, as it may on non-normal
    operators.) Both cells of the plan agree bit for bit; restart counts
    outside [0, 1000] are rejected."""
    torch = _torch()
    n = 64
    x = 1e-18 * 2.0 ** (np.arange(n) / 4)
    N0 = pg.grids.lognormal_ic(x, 20, 1.0, 1e12)
    t_q, bw_q = pg.quadrature.uniform(4)
    dt = 1.0
    for S0, m, bound in ((1.0, 4, 1e-11), (50.0, 12, 1e-8)):
        prm = pg.batch.cell_params(2, beta_br=6.73e-18, beta_sh=66.67, S0=S0,
                                   v_ref=float(x[n // 2]), alpha=1.0)
        agg = dict(kernel=5, beta_br=6.73e-18, beta_sh=66.67)
        brk = dict(t_q=t_q, bw_q=bw_q, selection=1, S0=S0, v_ref=float(x[n // 2]), alpha=1.0)
        dense = pyoracle.ros2_step(N0.copy(), x, dt, agg, brk)
        errs, res = [], []
        with pg.BatchPlan([x], [n, n], [0, 0], 5, 1, t_q, bw_q) as plan:
            assert plan.set_krylov_restarts(-1) == pg.ERR_INVALID_VALUE
            assert plan.set_krylov_restarts(1001) == pg.ERR_INVALID_VALUE
            for tol, restarts in ((0.0, 0), (1e-12, 10)):
                assert plan.set_krylov_tol(tol) == 0
                assert plan.set_krylov_restarts(restarts) == 0
                dN = t(np.concatenate([N0, N0]))
                resid = t(np.zeros(2))
                assert plan.ros2(dN, t(prm), dt, 1, krylov_dim=m, resid=resid) == 0
                torch.cuda.synchronize()
                a = dN.cpu().numpy()
                np.testing.assert_array_equal(a[:n].view(np.int64), a[n:].view(np.int64))
                errs.append(np.abs(a[:n] - dense).max() / np.abs(dense).max())
                res.append(float(resid.cpu().numpy().max()))
        assert res[0] > 1e-7 and errs[0] > 1e-4 * bound, (S0, errs, res)   # one cycle is not enough
        assert res[1] <= 1e-12, (S0, res)
        assert errs[1] < bound, (S0, errs)
