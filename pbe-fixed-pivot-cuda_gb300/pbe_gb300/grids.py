"""Pivot grids and initial distributions used by the workloads and tests.

Geometric grids are built from powers (x_i = x_0 * 2**(i/q)) so that every
pivot is within an ulp or two of the exact geometric value; the reference's
example helper builds them by repeated multiplication instead
(examples/common/pbe_examples_utils.hpp:83-90), which is offered as
`geometric_by_product` for parity tests of that construction.
"""
from __future__ import annotations

import math

import numpy as np


def geometric_pow2(n: int, x0: float, q: float) -> np.ndarray:
    """x_i = x0 * 2**(i/q), i < n."""
    i = np.arange(n, dtype=np.float64)
    return x0 * np.power(2.0, i / q)


def geometric_by_product(n: int, x0: float, r: float) -> np.ndarray:
    """x_0 = x0, x_i = x_{i-1} * r (pbe_examples_utils.hpp:83-90)."""
    x = np.empty(n)
    x[0] = x0
    for i in range(1, n):
        x[i] = x[i - 1] * r
    return x


def geometric_params(x: np.ndarray) -> tuple[float, float]:
    """(log_x0, inv_log_r) as the reference's callers pass them."""
    return math.log(x[0]), 1.0 / math.log(x[1] / x[0])


def lognormal_ic(x: np.ndarray, median_bin: int, sigma_ln: float, total: float,
                 cut: float = None) -> np.ndarray:
    """N_i proportional to exp(-(ln x_i - ln x_m)^2 / (2 sigma^2)) dln x, summed to `total`.
    (On a geometric grid dln x is constant, so it cancels in the normalisation.)
    cut: N_i = 0 exactly where |ln x_i - ln x_m| > cut sigma."""
    z = (np.log(x) - math.log(x[median_bin])) / sigma_ln
    N = np.exp(-0.5 * z * z)
    if cut is not None:
        N = np.where(np.abs(z) <= cut, N, 0.0)
    return N * (total / N.sum())


def exponential_ic(x: np.ndarray, N0: float, vc: float) -> np.ndarray:
    """Cell integrals of n(v) = N0/vc exp(-v/vc) over [x_i/sqrt(r), x_i sqrt(r)]
    on a geometric grid (pbe_examples_utils.hpp:120-136)."""
    sr = math.sqrt(x[1] / x[0])
    return N0 * (np.exp(-(x / sr) / vc) - np.exp(-(x * sr) / vc))


def config_n16384():
    """Single-instance workload: n = 16384 on x_i = 1e-21 * 2**(i/512) m^3,
    lognormal N (median bin 2048, sigma_ln = 1, total 1e14 m^-3),
    Brownian+shear beta_br = 6.73e-18, beta_sh = 4 G / 3 with G = 50 1/s,
    threshold selection S0 = 1e-3 1/s, v_min = x_8192."""
    n = 16384
    x = geometric_pow2(n, 1e-21, 512.0)
    N = lognormal_ic(x, 2048, 1.0, 1e14)
    return dict(n=n, x=x, N=N, beta_br=6.73e-18, beta_sh=4.0 * 50.0 / 3.0, S0=1e-3,
                v_min=float(x[8192]))


BATCH_SEED = 2026


def config_batched_cells(n_cells: int = 4096, seed: int = BATCH_SEED, n_max: int = 3840,
                         total: float = 1e13):
    """Batched-cell workload: `n_cells` independent cells, seeded
    (numpy.random.default_rng(seed)).
      sections n ~ U{64, 128, ..., n_max}; q ~ U{4, 8, 16, 32};
      grid x_i = 1e-21 * 2**(i/q) m^3 (one shared grid per q, n_max pivots;
      a cell uses its first n);
      Brownian + shear aggregation, beta_br = 6.73e-18 m^3/s,
      beta_sh = 4 G / 3 with G log-uniform in [10, 200] 1/s per cell;
      power-law selection S = S0 (x / x_ref)^a, S0 = 1e-3 1/s,
      a ~ U[0.5, 1.5], x_ref = the cell's middle pivot x[n // 2];
      uniform daughter on Gauss-Legendre 8 points;
      lognormal N (sigma_ln = 1, total `total` m^-3) with median at
      1e-18 m^3, or at bin n // 4 when the cell's grid ends below that, and
      exactly 0 beyond 5 sigma: on the coarse grids the upper bins reach
      volumes whose shear death rate times dt is far beyond RK4's stability
      limit (2.78), so they must start empty.
    Returns dict(grids, q_values, cell_n, cell_grid, params [n_cells, 8],
    N (packed), t_q, bw_q, seed)."""
    from .batch import cell_params
    from .quadrature import uniform

    rng = np.random.default_rng(seed)
    cell_n = 64 * rng.integers(1, n_max // 64 + 1, size=n_cells)
    q_values = np.array([4, 8, 16, 32])
    qi = rng.integers(0, 4, size=n_cells)
    G = np.exp(rng.uniform(math.log(10.0), math.log(200.0), size=n_cells))
    a = rng.uniform(0.5, 1.5, size=n_cells)
    grids = [geometric_pow2(n_max, 1e-21, float(q)) for q in q_values]
    x_ref = np.array([grids[g][n // 2] for g, n in zip(qi, cell_n)])
    params = cell_params(n_cells, beta0=0.0, beta_br=6.73e-18, beta_sh=4.0 * G / 3.0, S0=1e-3,
                         v_ref=x_ref, alpha=a)
    parts = []
    for g, n in zip(qi, cell_n):
        x = grids[g][:n]
        m = min(int(round(q_values[g] * math.log2(1e-18 / 1e-21))), n // 4)
        parts.append(lognormal_ic(x, m, 1.0, total, cut=5.0))
    t_q, bw_q = uniform(8)
    return dict(grids=grids, q_values=q_values, cell_n=cell_n.astype(np.int32),
                cell_grid=qi.astype(np.int32), params=params, N=np.concatenate(parts),
                t_q=t_q, bw_q=bw_q, seed=seed)


def config_flocculation_adjoint(n: int = 3840, n_steps: int = 200, switch_step: int = 100):
    """Two-stage flocculation adjoint workload: x_i = 1e-21 * 2**(i/128) m^3,
    Brownian + shear aggregation (beta_br = 6.73e-18 m^3/s, beta_sh = 4 G / 3
    with G = 100 1/s for steps < switch_step and 20 1/s after), power-law
    selection S0 = 5e-4 1/s, a = 1, v_ref = 1e-18 m^3, power-law daughter
    b(v|v') = 4 v^2 / v'^3 (exponent 2; 2 x 4 Gauss-Legendre points split at
    t = 1/2), dt = 0.5 s. Initial N: lognormal in ln x with median 3.2e-20 m^3
    (bin 640), sigma_ln = 1, total 1e12 m^-3, set to exactly 0 beyond 5 sigma
    (the upper bins have shear death rates far above 1/dt, so they start
    empty). Loss L = sum_i x_i^(2/3) N_i(T), so dL/dN(T) = x^(2/3).
    Returns dict(x, N0, t_q, bw_q, agg_sets (2), brk_sets (2), step_set, dt,
    n_steps, lam_T)."""
    from ._lib import AggregationParams, BreakageParams
    from .quadrature import power_law

    x = geometric_pow2(n, 1e-21, 128.0)
    N0 = lognormal_ic(x, min(640, n // 4), 1.0, 1e12, cut=5.0)
    t_q, bw_q = power_law(2.0, 4)
    agg = [AggregationParams(n=n, kernel_type=5, beta0=0.0, beta_br=6.73e-18,
                             beta_sh=4.0 * G / 3.0) for G in (100.0, 20.0)]
    brk = [BreakageParams(n=n, n_quad=len(t_q), selection=2, S0=5e-4, v_ref=1e-18, alpha=1.0,
                          v_min=0.0) for _ in range(2)]
    step_set = np.array([0 if s < switch_step else 1 for s in range(n_steps)], dtype=np.int32)
    return dict(x=x, N0=N0, t_q=t_q, bw_q=bw_q, agg_sets=agg, brk_sets=brk, step_set=step_set,
                dt=0.5, n_steps=n_steps, lam_T=x ** (2.0 / 3.0))


def config_batched_classes(n_cells: int = 512, seed: int = BATCH_SEED, width: int = 256,
                           total: float = 1e13):
    """Batched forward + adjoint workload with grids shared by size classes:
    `n_cells` cells (numpy.random.default_rng(seed)), n ~ U[256, 2048]; class
    k holds n in [256 k, 256 (k+1)) and shares one grid x_i = 1e-21 *
    2**(i/128) m^3 of 256 (k+1) pivots (class width `width`). Per-cell
    coefficients lognormal (sigma_ln = 0.5) around beta_br = 6.73e-18 m^3/s,
    beta_sh = 4 G / 3 with G = 50 1/s, S0 = 1e-3 1/s (power-law selection,
    a = 1, v_ref = 1e-18 m^3; uniform daughter, 4 Gauss-Legendre points).
    Lognormal N (median bin n // 4, sigma_ln = 1, total `total` m^-3, 0 beyond
    5 sigma).
    Returns dict(grids, cell_n, cell_grid, params, N, t_q, bw_q, seed)."""
    from .batch import cell_params
    from .quadrature import uniform

    rng = np.random.default_rng(seed)
    cell_n = rng.integers(256, 2049, size=n_cells)
    cls = np.minimum(cell_n // width, 2048 // width)
    classes = np.unique(cls)
    grids = [geometric_pow2(int(width * (k + 1)), 1e-21, 128.0) for k in classes]
    cell_grid = np.searchsorted(classes, cls).astype(np.int32)
    spread = lambda: np.exp(rng.normal(0.0, 0.5, size=n_cells))  # noqa: E731
    params = cell_params(n_cells, beta0=0.0, beta_br=6.73e-18 * spread(),
                         beta_sh=4.0 * 50.0 / 3.0 * spread(), S0=1e-3 * spread(), v_ref=1e-18,
                         alpha=1.0)
    N = np.concatenate([lognormal_ic(grids[g][:n], n // 4, 1.0, total, cut=5.0)
                        for g, n in zip(cell_grid, cell_n)])
    t_q, bw_q = uniform(4)
    return dict(grids=grids, cell_n=cell_n.astype(np.int32), cell_grid=cell_grid, params=params,
                N=N, t_q=t_q, bw_q=bw_q, seed=seed)
