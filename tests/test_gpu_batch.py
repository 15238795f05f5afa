"""Batched cells (pbe_batch_*): one persistent launch per RHS over many cells
with uneven section counts, RK4 steps as one CUDA graph.

Parity: every cell of a batch against the oracle's single-instance RHS on that
cell (same bound as the single-instance tests, |gpu - oracle| <= 1e-12 scale
+ 1e-280 with scale = the oracle's sum of |contributions|), and RK4 against
the oracle's rk4_step cell by cell."""
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


def mixed_batch(rng, kernel, selection, n_cells=40, n_max=300, kinds=("geo_fine", "geo_coarse",
                                                                         "generic", "geo_ref")):
    """Grids of several kinds (each n_max long) and cells with random n <= n_max
    (including n = 1, 2 and n_max), random N with zeros, per-cell coefficients."""
    grids = [make_grid(k, n_max, rng) for k in kinds]
    cell_grid = rng.integers(0, len(grids), size=n_cells)
    cell_n = rng.integers(1, n_max + 1, size=n_cells)
    cell_n[:4] = [1, 2, n_max, 12]
    N = [make_N("random", grids[g][:n], rng) for g, n in zip(cell_grid, cell_n)]
    k = [kk for kk in AGG_KERNELS if kk[0] == max(kernel, 0)][0]
    scale = np.exp(rng.uniform(-0.5, 0.5, size=n_cells))
    v_ref = np.array([grids[g][n // 2] for g, n in zip(cell_grid, cell_n)])
    params = pg.batch.cell_params(n_cells, beta0=k[1] * scale, beta_br=k[2] * scale,
                                  beta_sh=k[3] / scale, S0=1e-3 * scale, v_ref=v_ref,
                                  alpha=rng.uniform(0.5, 1.5, size=n_cells), v_min=v_ref)
    return grids, cell_n, cell_grid, N, params


def oracle_cell(Nc, x, kernel, selection, prm, t_q, bw_q):
    rhs = np.zeros(len(x))
    sc = np.zeros(len(x))
    if kernel >= 0:
        r, s, code = pyoracle.aggregation_rhs(Nc, x, kernel, prm[0], prm[1], prm[2],
                                              exact_bracket=True)
        assert code == 0
        rhs += r
        sc += s
    if selection >= 0:
        r, s, code = pyoracle.breakage_rhs(Nc, x, t_q, bw_q, selection, prm[3], prm[4], prm[5],
                                           prm[6])
        assert code == 0
        rhs += r
        sc += s
    return rhs, sc


def run_batch_rhs(plan, N, params, rhs0=None):
    torch = _torch()
    dN = t(np.concatenate(N))
    rhs = t(np.zeros(plan.total) if rhs0 is None else rhs0)
    dp = t(params)
    code = plan.rhs(dN, rhs, dp)
    torch.cuda.synchronize()
    return code, rhs.cpu().numpy()


@pytest.mark.parametrize("selection", [-1, 0, 2, 3])
@pytest.mark.parametrize("kernel", [-1, 0, 1, 2, 3, 4, 5])
def test_batch_rhs_matches_oracle_per_cell(kernel, selection):
    if kernel < 0 and selection < 0:
        pytest.skip("a plan needs aggregation or breakage")
    rng = np.random.default_rng(100 + 7 * kernel + selection)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, kernel, selection)
    t_q, bw_q = DAUGHTER
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel, selection, t_q, bw_q) as plan:
        code, rhs = run_batch_rhs(plan, N, params)
        assert code == 0, pg.error_string(code)
        for c, got in enumerate(plan.split(rhs)):
            x = grids[cell_grid[c]][:cell_n[c]]
            ref, sc = oracle_cell(N[c], x, kernel, selection, params[c], t_q, bw_q)
            assert_close(got, ref, sc, "batch k=%d sel=%d cell %d (n=%d)" % (kernel, selection, c,
                                                                           cell_n[c]))


def test_batch_rhs_accumulates_and_is_deterministic():
    rng = np.random.default_rng(5)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, 5, 2, n_cells=64)
    t_q, bw_q = DAUGHTER
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        base = rng.normal(size=plan.total)
        outs = [run_batch_rhs(plan, N, params, rhs0=base)[1] for _ in range(3)]
        for o in outs[1:]:
            assert np.array_equal(o.view(np.int64), outs[0].view(np.int64))
        _, plain = run_batch_rhs(plan, N, params)
        np.testing.assert_allclose(outs[0] - base, plain, rtol=1e-13, atol=1e-300 + 1e-15 * np.abs(base).max())


def test_batch_rhs_matches_single_instance_gpu():
    """Batched kernel vs the single-instance library calls on each cell."""
    torch = _torch()
    rng = np.random.default_rng(6)
    grids, cell_n, cell_grid, N, params = mixed_batch(rng, 5, 2, n_cells=24, n_max=2000,
                                                      kinds=("geo_fine", "generic"))
    t_q, bw_q = DAUGHTER
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        _, rhs = run_batch_rhs(plan, N, params)
        for c, got in enumerate(plan.split(rhs)):
            n = int(cell_n[c])
            x = grids[cell_grid[c]][:n]
            p = params[c]
            out = t(np.zeros(n))
            ap = pg.AggregationParams(n=n, kernel_type=5, beta0=p[0], beta_br=p[1], beta_sh=p[2])
            bp = pg.BreakageParams(n=n, n_quad=len(t_q), selection=2, S0=p[3], v_ref=p[4],
                                   alpha=p[5], v_min=p[6])
            tx, tN = t(x), t(N[c])
            assert pg.aggregation_rhs(tN, tx, out, ap) == 0
            assert pg.breakage_rhs(tN, tx, t(t_q), t(bw_q), out, bp) == 0
            torch.cuda.synchronize()
            ref = out.cpu().numpy()
            _, sc = oracle_cell(N[c], x, 5, 2, p, t_q, bw_q)
            assert_close(got, ref, sc, "batch vs single cell %d (n=%d)" % (c, n), tol=2e-12)


def test_batch_rk4_matches_oracle_rk4():
    torch = _torch()
    rng = np.random.default_rng(7)
    grids = [pg.grids.geometric_pow2(200, 1e-21, q) for q in (4.0, 16.0)]
    cell_n = np.array([200, 64, 1, 150, 37, 200, 128, 2])
    cell_grid = np.array([0, 1, 0, 1, 0, 1, 1, 0])
    N = [pg.grids.lognormal_ic(grids[g][:n], max(0, n // 4), 1.0, 1e13)
         for g, n in zip(cell_grid, cell_n)]
    G = rng.uniform(10, 200, size=len(cell_n))
    v_ref = np.array([grids[g][n // 2] for g, n in zip(cell_grid, cell_n)])
    params = pg.batch.cell_params(len(cell_n), beta0=0.0, beta_br=6.73e-18, beta_sh=4 * G / 3,
                                  S0=1e-3, v_ref=v_ref, alpha=rng.uniform(0.5, 1.5, len(cell_n)))
    t_q, bw_q = pg.quadrature.uniform(8)
    dt, steps = 0.5, 4
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        dN = t(np.concatenate(N))
        assert plan.rk4(dN, t(params), dt, steps) == 0
        torch.cuda.synchronize()
        got = plan.split(dN.cpu().numpy())
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        ref = N[c].copy()
        p = params[c]
        for _ in range(steps):
            ref = pyoracle.rk4_step(ref, x, dt,
                                    agg=dict(kernel=5, beta0=0.0, beta_br=p[1], beta_sh=p[2]),
                                    brk=dict(t_q=t_q, bw_q=bw_q, selection=2, S0=p[3], v_ref=p[4],
                                             alpha=p[5], v_min=p[6]))
        scale = np.abs(N[c]).max()
        np.testing.assert_allclose(got[c], ref, rtol=1e-11, atol=1e-11 * scale,
                                   err_msg="rk4 cell %d" % c)


def test_batch_rk4_graph_equals_percell_loop_and_reuses_graph():
    torch = _torch()
    cfg = pg.grids.config_batched_cells(n_cells=48, n_max=640)
    with pg.BatchPlan(cfg["grids"], cfg["cell_n"], cfg["cell_grid"], 5, 2, cfg["t_q"],
                      cfg["bw_q"]) as plan:
        dp = t(cfg["params"])
        a = t(cfg["N"])
        b = t(cfg["N"])
        c = t(cfg["N"])
        assert plan.rk4(a, dp, 0.5, 3) == 0
        assert plan.rk4(a, dp, 0.5, 3) == 0          # second launch of the cached graph
        assert plan.rk4(b, dp, 0.5, 6) == 0          # a new graph, six steps at once
        assert plan.rk4_percell(c, dp, 0.5, 6) == 0  # per-cell launch loop
        torch.cuda.synchronize()
        A, B, C = (v.cpu().numpy() for v in (a, b, c))
    assert np.array_equal(A.view(np.int64), B.view(np.int64))
    assert np.all(np.isfinite(A))
    np.testing.assert_allclose(A, C, rtol=1e-11, atol=1e-11 * np.abs(cfg["N"]).max())


def test_batch_autotune_schedule_and_results():
    torch = _torch()
    cfg = pg.grids.config_batched_cells(n_cells=96, n_max=1280)
    args = (cfg["grids"], cfg["cell_n"], cfg["cell_grid"], 5, 2, cfg["t_q"], cfg["bw_q"])
    with pg.BatchPlan(*args) as p0, pg.BatchPlan(*args, tune=True, retune=True) as p1:
        gs0, nb0 = p0.schedule()
        gs1, nb1 = p1.schedule()
        assert set(gs0) == set(gs1) and nb0 > 0 and nb1 > 0
        assert all(v in (32, 64, 128, 256) for v in gs1.values())
        dN, dp = t(cfg["N"]), t(cfg["params"])
        r0, r1 = t(np.zeros(p0.total)), t(np.zeros(p1.total))
        assert p0.rhs(dN, r0, dp) == 0 and p1.rhs(dN, r1, dp) == 0
        torch.cuda.synchronize()
        R0, R1 = r0.cpu().numpy(), r1.cpu().numpy()
    np.testing.assert_allclose(R1, R0, rtol=1e-12, atol=1e-12 * np.abs(R0).max())


def test_batch_plan_rejects_bad_input():
    g = [pg.grids.geometric_pow2(50, 1e-21, 8.0)]
    t_q, bw_q = DAUGHTER
    with pytest.raises(pg.PbeError) as e:
        pg.BatchPlan(g, [51], [0], 5)                       # more sections than the grid
    assert e.value.code == pg.ERR_INVALID_VALUE
    with pytest.raises(pg.PbeError):
        pg.BatchPlan(g, [10], [1], 5)                       # no such grid
    with pytest.raises(pg.PbeError):
        pg.BatchPlan(g, [10], [0], 5, 0, np.array([1.5]), np.array([1.0]))   # t_q > 1
    with pytest.raises(pg.PbeError):
        pg.BatchPlan([g[0][::-1]], [10], [0], 5)            # decreasing pivots
    with pytest.raises(pg.PbeError):
        pg.BatchPlan(g, [10], [0], -1, -1)                  # nothing to compute
    with pg.BatchPlan(g, [10, 20], [0, 0], 5) as plan:
        assert plan.rhs(0, 0, 0) == pg.ERR_INVALID_DEVICE_POINTER


@pytest.mark.parametrize("kernel,selection", [(3, -1), (-1, 2), (1, 0)])
def test_batch_rk4_single_term_plans_match_oracle(kernel, selection):
    """RK4 graph of plans with only aggregation, only breakage, or Sum +
    constant selection, against the oracle's rk4_step per cell."""
    import torch

    rng = np.random.default_rng(40 + kernel)
    grids = [pg.grids.geometric_pow2(120, 1e-21, 8.0), make_grid("generic", 120, rng)]
    cell_n = np.array([120, 37, 1, 90])
    cell_grid = np.array([0, 1, 0, 1])
    N = [pg.grids.lognormal_ic(grids[g][:n], max(0, n // 4), 1.0, 1e12, cut=5.0)
         for g, n in zip(cell_grid, cell_n)]
    k = [kk for kk in AGG_KERNELS if kk[0] == max(kernel, 0)][0]
    v_ref = np.array([grids[g][n // 2] for g, n in zip(cell_grid, cell_n)])
    # coefficients that keep every rate well inside RK4's stability region
    params = pg.batch.cell_params(len(cell_n), beta0=1e-20, beta_br=k[2], beta_sh=k[3],
                                  S0=1e-3, v_ref=v_ref, alpha=1.2)
    t_q, bw_q = pg.quadrature.uniform(4)
    dt, steps = 0.5, 3
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel, selection, t_q, bw_q) as plan:
        dN = t(np.concatenate(N))
        assert plan.rk4(dN, t(params), dt, steps) == 0
        torch.cuda.synchronize()
        got = plan.split(dN.cpu().numpy())
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        p = params[c]
        ref = N[c].copy()
        agg = dict(kernel=kernel, beta0=p[0], beta_br=p[1], beta_sh=p[2]) if kernel >= 0 else None
        brk = (dict(t_q=t_q, bw_q=bw_q, selection=selection, S0=p[3], v_ref=p[4], alpha=p[5],
                    v_min=p[6]) if selection >= 0 else None)
        for _ in range(steps):
            ref = pyoracle.rk4_step(ref, x, dt, agg=agg, brk=brk)
        np.testing.assert_allclose(got[c], ref, rtol=1e-11, atol=1e-11 * np.abs(N[c]).max(),
                                   err_msg="k=%d sel=%d cell %d" % (kernel, selection, c))


def test_config1_constant_kernel_rk4_follows_scott_and_the_oracle():
    """The reference's CPU-runnable case: constant kernel beta0 = 1e-15 on
    x_i = 1e-18 2^i (n = 256), N_i = N0 (x_i/x_m) e^(-x_i/x_m) dx_i/x_m,
    1000 RK4 steps of dt = 1 s as one graph. Total number follows
    Smoluchowski/Scott M0(t) = M0(0) / (1 + beta0 M0(0) t / 2)
    (pbe_examples_utils.hpp:207-221) to 1e-9, and every bin follows the
    oracle's 1000 rk4_step calls (1e-10 of the largest N)."""
    import torch

    n = 256
    x = 1e-18 * np.power(2.0, np.arange(n, dtype=np.float64))
    xm, N0, b0 = 4e-18, 1e12, 1e-15
    dx = x * np.sqrt(2.0) - x / np.sqrt(2.0)
    N = N0 * (x / xm) * np.exp(-x / xm) * dx / xm
    params = pg.batch.cell_params(1, beta0=b0)
    steps = 1000
    with pg.BatchPlan([x], [n], [0], 0) as plan:
        dN = t(N.copy())
        assert plan.rk4(dN, t(params), 1.0, steps) == 0
        torch.cuda.synchronize()
        got = dN.cpu().numpy()
    M0 = N.sum()
    expect = M0 / (1.0 + b0 * M0 * steps / 2.0)
    assert abs(got.sum() - expect) / expect < 1e-9
    ref = N.copy()
    agg = dict(kernel=0, beta0=b0)
    for _ in range(steps):
        ref = pyoracle.rk4_step(ref, x, 1.0, agg=agg)
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-10 * np.abs(ref).max())


def test_breakage_gather_modes_are_bitwise_equal():
    """The breakage term gathered by the per-cell prep CTA or by the pair
    tasks (for their own bins) uses the same lanes, loops and butterfly: RHS,
    Jacobian-vector product and RK4 steps agree bit for bit, with lag chunks
    (few tiles) and without, on geometric and generic grids. Conflicting or
    unknown plan flags are rejected."""
    torch = _torch()
    rng = np.random.default_rng(77)
    t_q, bw_q = DAUGHTER
    for n_cells in (24, 160):            # lag chunks (few tiles), then none
        grids, cell_n, cell_grid, N, params = mixed_batch(rng, 5, 2, n_cells=n_cells, n_max=400)
        N = [np.abs(Nc) for Nc in N]
        v = [rng.standard_normal(len(Nc)) * Nc for Nc in N]
        outs = {}
        for mode in ("prep", "tasks"):
            with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q,
                              breakage_gather=mode) as plan:
                dN, dv, dp = t(np.concatenate(N)), t(np.concatenate(v)), t(params)
                r = torch.zeros_like(dN)
                jv = torch.zeros_like(dN)
                assert plan.rhs(dN, r, dp) == 0
                assert plan.jvp(dN, dv, jv, dp) == 0
                Y = dN.clone()
                assert plan.rk4(Y, dp, 0.25, 3) == 0
                torch.cuda.synchronize()
                outs[mode] = [a.cpu().numpy() for a in (r, jv, Y)]
        for a, b in zip(outs["prep"], outs["tasks"]):
            np.testing.assert_array_equal(a.view(np.int64), b.view(np.int64))
    lib = pg.load()
    import ctypes

    h = ctypes.c_void_p()
    g = np.ascontiguousarray(grids[0], dtype=np.float64)
    gn = np.array([len(g)], dtype=np.int32)
    cn = np.array([len(g)], dtype=np.int32)
    cg = np.zeros(1, dtype=np.int32)
    for flags in (pg.BATCH_BRK_PREP | pg.BATCH_BRK_TASKS, 64):
        code = lib.pbe_batch_create(ctypes.byref(h), 1, gn.ctypes.data, g.ctypes.data, 1,
                                    cn.ctypes.data, cg.ctypes.data, 5, -1, 0, None, None,
                                    flags, None)
        assert code == pg.ERR_INVALID_VALUE
