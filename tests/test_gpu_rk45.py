"""Adaptive embedded Dormand-Prince 5(4) on the batched plan (pbe_batch_rk45):
accuracy against the oracle's fixed-step RK4 with a step 100 times smaller
than the adaptive steps, per-cell step sizes (a faster cell takes more steps),
determinism, and the not-ready return when the attempt budget runs out.
The oracle reference uses 20 RK4 steps for every accepted adaptive step
(at least 200); bound 1e-6 relative + 1e-7 of the cell's largest N."""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import t

pytestmark = pytest.mark.gpu


def batch(n_cells=6, n=96):
    """Cells 0 and 1 are identical except that every rate of cell 1 is 30 times
    larger (so over the same interval it goes through 30 times more of its
    evolution); the others differ in grid, n and coefficients."""
    rng = np.random.default_rng(21)
    grids = [pg.grids.geometric_pow2(n, 1e-21, 8.0), pg.grids.geometric_pow2(n, 1e-20, 16.0)]
    cell_grid = np.arange(n_cells) % 2
    cell_grid[1] = cell_grid[0]
    cell_n = rng.integers(n // 2, n + 1, size=n_cells)
    cell_n[1] = cell_n[0]
    N = [pg.grids.lognormal_ic(grids[g][:m], m // 4, 1.0, 1e13, cut=5.0) for g, m in zip(cell_grid, cell_n)]
    G = rng.uniform(20.0, 100.0, size=n_cells)
    G[1] = G[0]
    scale = np.ones(n_cells)
    scale[1] = 30.0
    v_ref = np.array([grids[g][m // 2] for g, m in zip(cell_grid, cell_n)])
    params = pg.batch.cell_params(n_cells, beta0=0.0, beta_br=6.73e-18 * scale,
                                  beta_sh=4 * G / 3 * scale, S0=1e-3 * scale, v_ref=v_ref, alpha=1.0)
    t_q, bw_q = pg.quadrature.uniform(4)
    return grids, cell_n, cell_grid, N, params, t_q, bw_q


def test_rk45_matches_fine_rk4_oracle_and_adapts_per_cell():
    import torch

    grids, cell_n, cell_grid, N, params, t_q, bw_q = batch()
    t_end = 40.0
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        dN = t(np.concatenate(N))
        code, steps, rejects, att = plan.rk45(dN, t(params), t_end, rtol=1e-10, atol=1e-3, dt0=0.1)
        torch.cuda.synchronize()
        assert code == 0, pg.error_string(code)
        got = plan.split(dN.cpu().numpy())
    assert steps[1] > steps[0]                # the same cell at 30x the rates needs more steps
    for c in range(len(cell_n)):
        x = grids[cell_grid[c]][:cell_n[c]]
        p = params[c]
        ref = N[c].copy()
        nfine = max(200, 20 * int(steps[c]))
        for _ in range(nfine):
            ref = pyoracle.rk4_step(ref, x, t_end / nfine,
                                    agg=dict(kernel=5, beta0=0.0, beta_br=p[1], beta_sh=p[2]),
                                    brk=dict(t_q=t_q, bw_q=bw_q, selection=2, S0=p[3], v_ref=p[4],
                                             alpha=p[5], v_min=p[6]))
        scale = np.abs(N[c]).max()
        np.testing.assert_allclose(got[c], ref, rtol=1e-6, atol=1e-7 * scale,
                                   err_msg="cell %d (%d steps)" % (c, steps[c]))


def test_rk45_is_deterministic_and_reports_budget_exhaustion():
    import torch

    grids, cell_n, cell_grid, N, params, t_q, bw_q = batch(n_cells=4, n=64)
    with pg.BatchPlan(grids, cell_n, cell_grid, 5, 2, t_q, bw_q) as plan:
        outs = []
        for _ in range(2):
            dN = t(np.concatenate(N))
            code, steps, _, _ = plan.rk45(dN, t(params), 20.0, rtol=1e-9, atol=1e-3, dt0=0.05)
            assert code == 0
            torch.cuda.synchronize()
            outs.append((dN.cpu().numpy(), steps.copy()))
        assert np.array_equal(outs[0][0].view(np.int64), outs[1][0].view(np.int64))
        assert np.array_equal(outs[0][1], outs[1][1])
        dN = t(np.concatenate(N))
        code, steps, _, att = plan.rk45(dN, t(params), 20.0, rtol=1e-12, atol=1e-6, dt0=1e-3,
                                        max_attempts=3)
        assert code == pg.ERR_NOT_READY and att == 3
        assert plan.rk45(dN, t(params), -1.0)[0] == pg.ERR_INVALID_VALUE
