"""The batched plans the benchmark times, checked against the oracle.

bench.py credits two batched workloads:
  * 4096 cells (pbe_gb300.grids.config_batched_cells, seed 2026): n from 64 to
    3840, four geometric grids with q = 4, 8, 16, 32 pivots per octave (the
    q = 4 grid spans 960 octaves), per-cell shear rate, power-law selection,
    uniform GL8 daughter, autotuned schedule;
  * 512 cells sharing grids by size class (config_batched_classes).
Here the same plans (built the same way, tune=True) run one RHS and one RK4
step on the GPU, and sampled cells are compared with the serial oracle:
the largest cell, the smallest, the largest coarse (q = 4) cell, one cell per
q, and cells spread over the rest -- RHS per bin at |gpu - oracle| <= 1e-12 *
scale + 1e-280 (scale = the oracle's sum of |contributions|, as every parity
test here), RK4 at rtol 1e-11 (the batched RK4 tests' bound).
"""
import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import assert_close, t

pytestmark = pytest.mark.gpu


def _oracle_rhs(Nc, x, prm, t_q, bw_q):
    r1, s1, c1 = pyoracle.aggregation_rhs(Nc, x, pg.AGG_BROWNIAN_SHEAR, prm[0], prm[1], prm[2],
                                          exact_bracket=True)
    r2, s2, c2 = pyoracle.breakage_rhs(Nc, x, t_q, bw_q, pg.SEL_POWERLAW, prm[3], prm[4], prm[5],
                                       prm[6])
    assert c1 == 0 and c2 == 0
    return r1 + r2, s1 + s2


def _oracle_rk4(Nc, x, prm, t_q, bw_q, dt):
    return pyoracle.rk4_step(Nc, x, dt,
                             agg=dict(kernel=pg.AGG_BROWNIAN_SHEAR, beta0=prm[0], beta_br=prm[1],
                                      beta_sh=prm[2]),
                             brk=dict(t_q=t_q, bw_q=bw_q, selection=pg.SEL_POWERLAW, S0=prm[3],
                                      v_ref=prm[4], alpha=prm[5], v_min=prm[6]))


def _sample_cells(cell_n, cell_grid, q_of_grid, rng, extra):
    """Largest, smallest, largest coarsest-grid cell, one per grid, plus `extra` random."""
    pick = [int(np.argmax(cell_n)), int(np.argmin(cell_n))]
    coarse = np.flatnonzero(q_of_grid[cell_grid] == q_of_grid.min())
    pick.append(int(coarse[np.argmax(cell_n[coarse])]))
    for g in range(len(q_of_grid)):
        members = np.flatnonzero(cell_grid == g)
        if len(members):
            pick.append(int(rng.choice(members)))
    pick += [int(c) for c in rng.choice(len(cell_n), size=extra, replace=False)]
    return sorted(set(pick))


def _check_plan(cfg, q_of_grid, extra, rk4_cells):
    import torch

    grids, cell_n, cell_grid = cfg["grids"], cfg["cell_n"], cfg["cell_grid"]
    t_q, bw_q, P = cfg["t_q"], cfg["bw_q"], cfg["params"]
    off = np.r_[0, np.cumsum(cell_n)]
    rng = np.random.default_rng(11)
    cells = _sample_cells(cell_n, cell_grid, q_of_grid, rng, extra)
    dt = 0.5
    with pg.BatchPlan(grids, cell_n, cell_grid, pg.AGG_BROWNIAN_SHEAR, pg.SEL_POWERLAW, t_q,
                      bw_q, tune=True) as plan:
        dN, dP = t(cfg["N"]), t(P)
        out = t(np.zeros(plan.total))
        assert plan.rhs(dN, out, dP) == 0
        Y = dN.clone()
        assert plan.rk4(Y, dP, dt, 1) == 0
        torch.cuda.synchronize()
        rhs = out.cpu().numpy()
        Y1 = Y.cpu().numpy()
    worst = 0.0
    for c in cells:
        x = grids[cell_grid[c]][:cell_n[c]]
        Nc = cfg["N"][off[c]:off[c + 1]]
        ref, sc = _oracle_rhs(Nc, x, P[c], t_q, bw_q)
        got = rhs[off[c]:off[c + 1]]
        assert_close(got, ref, sc, "bench plan cell %d (n=%d, grid %d)" % (c, cell_n[c], cell_grid[c]))
        worst = max(worst, float(np.max(np.abs(got - ref) / np.maximum(sc, 1e-300))))
    for c in cells[:rk4_cells]:
        x = grids[cell_grid[c]][:cell_n[c]]
        Nc = cfg["N"][off[c]:off[c + 1]]
        ref = _oracle_rk4(Nc, x, P[c], t_q, bw_q, dt)
        np.testing.assert_allclose(Y1[off[c]:off[c + 1]], ref, rtol=1e-11,
                                   atol=1e-11 * np.abs(Nc).max(), err_msg="rk4 cell %d" % c)
    return cells, worst


def test_config3_bench_plan_matches_oracle():
    cfg = pg.grids.config_batched_cells()
    cells, worst = _check_plan(cfg, np.asarray(cfg["q_values"]), extra=8, rk4_cells=6)
    assert len(cells) >= 12
    n_of = cfg["cell_n"][cells]
    assert n_of.max() == cfg["cell_n"].max() and n_of.min() == cfg["cell_n"].min()
    print("config 3 plan: %d cells checked (n %s), worst |gpu-oracle|/scale %.2e"
          % (len(cells), list(map(int, n_of)), worst))


def test_config5_classes_plan_matches_oracle():
    cfg = pg.grids.config_batched_classes()
    q_of_grid = np.array([len(g) for g in cfg["grids"]], dtype=float)   # every grid q = 128
    cells, worst = _check_plan(cfg, q_of_grid, extra=6, rk4_cells=4)
    assert len(cells) >= 12
    print("config 5 plan: %d cells checked, worst |gpu-oracle|/scale %.2e" % (len(cells), worst))
