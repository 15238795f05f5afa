"""Batched VJP (pbe_batch_rhs_vjp) and batched RK4 tape (pbe_batch_tape_*).

The batched VJP is checked cell by cell against the oracle's adjoint (same
bound as the single-instance VJP tests: |gpu - oracle| <= 1e-12 s + 1e-280
with the oracle's per-entry scales); the batched tape against the
single-instance tape run cell by cell (which test_gpu_adjoint.py pins to the
oracle and to finite differences), for independence of the checkpoint
interval, and against central differences of an L2 misfit."""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import AGG_KERNELS, assert_close, make_grid, make_N, t

pytestmark = pytest.mark.gpu

DAUGHTER = pg.quadrature.uniform(4)


def _torch():
    import torch

    return torch


def mixed(rng, kernel, n_cells=30, n_max=240):
    grids = [make_grid(k, n_max, rng) for k in ("geo_fine", "geo_coarse", "generic")]
    cell_grid = rng.integers(0, len(grids), size=n_cells)
    cell_n = rng.integers(1, n_max + 1, size=n_cells)
    cell_n[:3] = [1, 2, n_max]
    N = [make_N("random", grids[g][:n], rng) for g, n in zip(cell_grid, cell_n)]
    lam = [rng.normal(size=n) for n in cell_n]
    k = [kk for kk in AGG_KERNELS if kk[0] == max(kernel, 0)][0]
    sc = np.exp(rng.uniform(-0.5, 0.5, size=n_cells))
    v_ref = np.array([grids[g][n // 2] for g, n in zip(cell_grid, cell_n)])
    params = pg.batch.cell_params(n_cells, beta0=k[1] * sc, beta_br=k[2] * sc, beta_sh=k[3] / sc,
                                  S0=1e-3 * sc, v_ref=v_ref, alpha=rng.uniform(0.5, 1.5, n_cells),
                                  v_min=v_ref)
    return grids, cell_n, cell_grid, N, lam, params


@pytest.mark.parametrize("selection", [-1, 0, 2, 3])
@pytest.mark.parametrize("kernel", [-1, 0, 1, 2, 3, 4, 5])
def test_batch_vjp_matches_oracle_per_cell(kernel, selection):
    if kernel < 0 and selection < 0:
        pytest.skip("a plan needs aggregation or breakage")
    torch = _torch()
    rng = np.random.default_rng(300 + 7 * kernel + selection)
    grids, cell_n, cell_grid, N, lam, params = mixed(rng, kernel)
    t_q, bw_q = DAUGHTER
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel, selection, t_q, bw_q) as plan:
        gN = t(np.zeros(plan.total))
        gp = t(np.zeros((len(cell_n), 8)))
        assert plan.rhs_vjp(t(np.concatenate(N)), t(np.concatenate(lam)), gN, gp, t(params)) == 0
        torch.cuda.synchronize()
        gN = plan.split(gN.cpu().numpy())
        gp = gp.cpu().numpy()
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        p = params[c]
        rN, sN = np.zeros(len(x)), np.zeros(len(x))
        rp, sp = np.zeros(8), np.zeros(8)
        if kernel >= 0:
            a, ap, sa, sap, _ = pyoracle.aggregation_rhs_vjp(N[c], x, lam[c], kernel, p[0], p[1],
                                                             p[2], exact_bracket=True,
                                                             with_scale=True)
            rN += a; sN += sa; rp[:3] += ap; sp[:3] += sap
        if selection >= 0:
            b, bp, sb, sbp, _ = pyoracle.breakage_rhs_vjp(N[c], x, t_q, bw_q, lam[c], selection,
                                                          p[3], p[4], p[5], p[6], with_scale=True)
            rN += b; sN += sb; rp[3:7] += bp; sp[3:7] += sbp
        what = "k=%d sel=%d cell %d n=%d" % (kernel, selection, c, cell_n[c])
        assert_close(gN[c], rN, sN, "dL/dN " + what)
        assert_close(gp[c, :7], rp[:7], sp[:7], "dL/dparams " + what)


def floc_batch(n_cells=10, n=160):
    rng = np.random.default_rng(11)
    grids = [pg.grids.geometric_pow2(n, 1e-21, 16.0)]
    cell_n = rng.integers(n // 3, n + 1, size=n_cells)
    cell_n[0] = n
    cell_grid = np.zeros(n_cells, dtype=int)
    N = np.concatenate([pg.grids.lognormal_ic(grids[0][:m], m // 4, 1.0, 1e13, cut=5.0)
                        for m in cell_n])
    params = pg.batch.cell_params(n_cells, beta0=0.0, beta_br=6.73e-18 * rng.uniform(0.8, 1.2, n_cells),
                                  beta_sh=4 * 50 / 3 * rng.uniform(0.8, 1.2, n_cells),
                                  S0=5e-4 * rng.uniform(0.8, 1.2, n_cells), v_ref=1e-19, alpha=1.0)
    t_q, bw_q = pg.quadrature.power_law(2.0, 4)
    return grids, cell_n, cell_grid, N, params, t_q, bw_q


def batch_tape(plan, N, params, dt, steps, every, lam_fn):
    torch = _torch()
    dN = t(N)
    dp = t(params)
    assert plan.tape_forward(dN, dp, dt, steps, every) == 0
    lam = lam_fn(dN)
    gN0 = t(np.zeros(plan.total))
    gp = t(np.zeros((plan.n_cells, 8)))
    assert plan.tape_backward(lam, gN0, gp) == 0
    torch.cuda.synchronize()
    return dN.cpu().numpy(), gN0.cpu().numpy(), gp.cpu().numpy()


def test_batch_tape_matches_single_instance_tapes():
    grids, cell_n, cell_grid, N, params, t_q, bw_q = floc_batch()
    dt, steps = 0.5, 7
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        x_all = np.concatenate([grids[0][:m] for m in cell_n])
        w = t(x_all ** (2.0 / 3.0))
        NT, gN0, gp = batch_tape(plan, N, params, dt, steps, 3, lambda dN: w)
        NTc, gNc = plan.split(NT), plan.split(gN0)
        offs = plan.offsets
    for c in range(len(cell_n)):
        n = int(cell_n[c])
        x = grids[0][:n]
        p = params[c]
        agg = [pg.AggregationParams(n=n, kernel_type=5, beta0=0.0, beta_br=p[1], beta_sh=p[2])]
        brk = [pg.BreakageParams(n=n, n_quad=len(t_q), selection=2, S0=p[3], v_ref=p[4], alpha=p[5])]
        torch = _torch()
        with pg.Rk4Tape(steps, dt, 3, agg, brk) as tape:
            Nc = t(N[offs[c]:offs[c + 1]])
            tx, ttq, tbw = t(x), t(t_q), t(bw_q)     # the tape keeps these until backward
            assert tape.forward(Nc, tx, ttq, tbw) == 0
            g0 = t(np.zeros(n))
            ga, gb = t(np.zeros(3)), t(np.zeros(4))
            assert tape.backward(t(x ** (2.0 / 3.0)), g0, ga, gb) == 0
            torch.cuda.synchronize()
        np.testing.assert_allclose(NTc[c], Nc.cpu().numpy(), rtol=1e-12, atol=1e-300)
        ref = g0.cpu().numpy()
        np.testing.assert_allclose(gNc[c], ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
        np.testing.assert_allclose(gp[c, 1:3], ga.cpu().numpy()[1:3], rtol=1e-9)
        np.testing.assert_allclose(gp[c, [3, 5]], gb.cpu().numpy()[[0, 2]], rtol=1e-9)


def test_batch_tape_checkpoint_interval_is_bitwise_neutral():
    grids, cell_n, cell_grid, N, params, t_q, bw_q = floc_batch(n_cells=6, n=100)
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        lam = t(np.random.default_rng(2).normal(size=plan.total))
        outs = [batch_tape(plan, N, params, 0.5, 6, every, lambda dN: lam) for every in (1, 4, 6, 50)]
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_batch_tape_l2_misfit_matches_finite_differences():
    """L = 1/2 |N(T) - N*(T)|^2 with N* from perturbed coefficients; central
    differences (h = 1e-6 relative) of the batched forward."""
    torch = _torch()
    grids, cell_n, cell_grid, N, params, t_q, bw_q = floc_batch(n_cells=8, n=120)
    dt, steps = 0.5, 8
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        target = params.copy()
        target[:, 1] *= 1.05
        target[:, 2] *= 0.95
        Nstar = t(N)
        assert plan.rk4(Nstar, t(target), dt, steps) == 0

        def run(prm, N0=N):
            dN = t(N0)
            assert plan.rk4(dN, t(prm), dt, steps) == 0
            torch.cuda.synchronize()
            return dN

        def L(prm, N0=N):
            r = run(prm, N0) - Nstar
            return 0.5 * float((r * r).sum())

        NT, gN0, gp = batch_tape(plan, N, params, dt, steps, 3, lambda dN: dN - Nstar)
        L0 = abs(L(params))
        for c, j in ((0, 1), (0, 2), (3, 2), (5, 3), (7, 5)):
            h = 1e-6 * params[c, j]
            pp, pm = params.copy(), params.copy()
            pp[c, j] += h
            pm[c, j] -= h
            fd = (L(pp) - L(pm)) / (2 * h)
            assert abs(fd - gp[c, j]) <= 2e-6 * abs(gp[c, j]) + 1e-12 * L0 / h, (c, j, fd, gp[c, j])
        for m in (5, 40, int(plan.offsets[3]) + 10):
            h = 1e-6 * N[m]
            Np, Nm = N.copy(), N.copy()
            Np[m] += h
            Nm[m] -= h
            fd = (L(params, Np) - L(params, Nm)) / (2 * h)
            assert abs(fd - gN0[m]) <= 2e-6 * abs(gN0[m]) + 1e-12 * L0 / h, (m, fd, gN0[m])
