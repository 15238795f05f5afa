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


def lognormal_ic(x: np.ndarray, median_bin: int, sigma_ln: float, total: float) -> np.ndarray:
    """N_i proportional to exp(-(ln x_i - ln x_m)^2 / (2 sigma^2)) dln x, summed to `total`.
    (On a geometric grid dln x is constant, so it cancels in the normalisation.)"""
    z = (np.log(x) - math.log(x[median_bin])) / sigma_ln
    N = np.exp(-0.5 * z * z)
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
