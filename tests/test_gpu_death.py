"""Death term of batched cells: the FP64 tensor-core GEMM (mma.sync f64) and
the moment form against a direct sum over k of beta(x_i, x_k) N_k (numpy,
pair by pair), for every kernel type, cells of uneven n sharing grids.
Bound: |gpu - ref| <= 1e-12 sum_k |beta N_i N_k| + 1e-280."""
import numpy as np
import pytest

import pbe_gb300 as pg
from gpu_util import t

pytestmark = pytest.mark.gpu


def beta(kernel, xi, xk, p):
    ai, ak = np.cbrt(xi), np.cbrt(xk)
    if kernel == 0:
        return p[0] * np.ones_like(xi * xk)
    if kernel == 1:
        return p[0] * (xi + xk)
    if kernel == 2:
        return p[0] * xi * xk
    b = 0.0
    if kernel in (3, 5):
        b = b + p[1] * (ai / ak + ak / ai + 2.0)
    if kernel in (4, 5):
        b = b + p[2] * (ai + ak) ** 3
    return b


@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 4, 5])
def test_death_gemm_and_moments_match_direct_sum(kernel):
    import torch

    rng = np.random.default_rng(40 + kernel)
    grids = [pg.grids.geometric_pow2(200, 1e-21, 16.0), pg.grids.geometric_pow2(130, 1e-19, 4.0)]
    n_cells = 150                                   # > 64 per grid: several row tiles
    cell_grid = rng.integers(0, 2, size=n_cells)
    cell_n = np.array([rng.integers(1, len(grids[g]) + 1) for g in cell_grid])
    cell_n[:3] = [1, 200 if cell_grid[1] == 0 else 130, 65]
    cell_n = np.minimum(cell_n, [len(grids[g]) for g in cell_grid])
    N = [rng.lognormal(20.0, 2.0, size=n) for n in cell_n]
    scale = np.exp(rng.uniform(-0.5, 0.5, size=n_cells))
    params = pg.batch.cell_params(n_cells, beta0=1e-15 * scale, beta_br=6.73e-18 * scale,
                                  beta_sh=66.7 / scale)
    with pg.BatchPlan(grids, cell_n, cell_grid, kernel) as plan:
        dN, dp = t(np.concatenate(N)), t(params)
        outs = {}
        for method in (pg.DEATH_MOMENTS, pg.DEATH_DMMA):
            out = t(np.full(plan.total, np.nan))
            assert plan.death(dN, out, dp, method) == 0
            torch.cuda.synchronize()
            outs[method] = plan.split(out.cpu().numpy())
    for c in range(n_cells):
        x = grids[cell_grid[c]][:cell_n[c]]
        B = beta(kernel, x[:, None], x[None, :], params[c])
        terms = B * N[c][None, :] * N[c][:, None]
        ref = terms.sum(axis=1)
        lim = 1e-12 * np.abs(terms).sum(axis=1) + 1e-280
        for method, name in ((pg.DEATH_MOMENTS, "moments"), (pg.DEATH_DMMA, "dmma")):
            err = np.abs(outs[method][c] - ref)
            assert np.all(err <= lim), (name, c, int(np.argmax(err / lim)), float((err / lim).max()))


def test_death_needs_aggregation_and_valid_method():
    g = [pg.grids.geometric_pow2(20, 1e-21, 4.0)]
    t_q, bw_q = pg.quadrature.uniform(2)
    with pg.BatchPlan(g, [20], [0], -1, 0, t_q, bw_q) as plan:
        z = t(np.zeros(20))
        assert plan.death(z, z, t(np.zeros((1, 8)))) == pg.ERR_INVALID_VALUE
    with pg.BatchPlan(g, [20], [0], 5) as plan:
        z = t(np.zeros(20))
        assert plan.death(z, z, t(np.zeros((1, 8))), method=7) == pg.ERR_INVALID_VALUE
