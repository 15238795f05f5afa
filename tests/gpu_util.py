"""Helpers shared by the GPU tests: run the library through the C ABI on numpy
inputs and compare with the oracle bin by bin.

Tolerance (stated once, used everywhere):
    |gpu_i - oracle_i| <= TOL * scale_i + ABS_FLOOR
with scale_i = sum of |contributions| the oracle deposited into bin i, so the
bound stays meaningful where birth and death cancel. TOL = 1e-12.
ABS_FLOOR = 1e-280: once a pair rate beta N_j N_k approaches the subnormal
range (< 2.2e-308) every implementation, the reference included, loses its
relative precision there, so bins whose values are that small are compared
absolutely. Physical number densities are many decades above it.
"""
from __future__ import annotations

import math

import numpy as np

import pbe_gb300 as pg
import pyoracle

TOL = 1e-12
ABS_FLOOR = 1e-280


def dev():
    import torch

    return torch.device("cuda:0")


def t(a):
    import torch

    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev())


def agg_params(n, kernel, b0, bbr, bsh, x=None, geometric=True):
    p = pg.AggregationParams(n=n, kernel_type=kernel, beta0=b0, beta_br=bbr, beta_sh=bsh)
    if x is not None and geometric and n >= 2:
        p.log_x0, p.inv_log_r = math.log(x[0]), 1.0 / math.log(x[1] / x[0])
    return p


def gpu_agg(N, x, p, mode=pg.MODE_DEFAULT, rhs0=None, stream=None):
    import torch

    rhs = t(np.zeros(len(x)) if rhs0 is None else rhs0)
    code = pg.aggregation_rhs(t(N), t(x), rhs, p, stream=stream, mode=mode)
    torch.cuda.synchronize()
    return code, rhs.cpu().numpy()


def gpu_brk(N, x, t_q, bw_q, p, mode=pg.MODE_DEFAULT, rhs0=None):
    import torch

    rhs = t(np.zeros(len(x)) if rhs0 is None else rhs0)
    code = pg.breakage_rhs(t(N), t(x), t(t_q), t(bw_q), rhs, p, mode=mode)
    torch.cuda.synchronize()
    return code, rhs.cpu().numpy()


def oracle_agg(N, x, p):
    """Oracle with the exact bracket x[lo] <= x_j + x_k < x[lo+1] (the library's
    bracket on every grid; see oracle_agg_reference for the reference's)."""
    return pyoracle.aggregation_rhs(N, x, p.kernel_type, p.beta0, p.beta_br, p.beta_sh, p.log_x0,
                                    p.inv_log_r, exact_bracket=True)


def oracle_agg_reference(N, x, p):
    """Oracle following the reference literally (logarithm bracket on geometric
    grids). Returns (rhs, scale, misplaced): `misplaced` bounds, per bin, what
    the reference's near-tie bracket choices move relative to the exact bracket."""
    ref, scale, mis, _ = pyoracle.aggregation_rhs(N, x, p.kernel_type, p.beta0, p.beta_br,
                                                  p.beta_sh, p.log_x0, p.inv_log_r,
                                                  exact_bracket=False, with_misplaced=True)
    return ref, scale, mis


def oracle_brk(N, x, t_q, bw_q, p):
    return pyoracle.breakage_rhs(N, x, t_q, bw_q, p.selection, p.S0, p.v_ref, p.alpha, p.v_min)


def assert_close(got, ref, scale, what="", tol=TOL, extra=None):
    """|got - ref| <= tol * scale + ABS_FLOOR (+ extra, the reference's measured
    near-tie misplacement, when comparing against the reference's own bracket)."""
    same_inf = np.isinf(got) & (got == ref)    # both overflowed the same way
    err = np.where(same_inf, 0.0, np.abs(got - ref))
    lim = tol * np.where(np.isinf(scale), 0.0, scale) + ABS_FLOOR
    if extra is not None:
        lim = lim + 1.000001 * extra
    bad = ~(err <= lim)   # NaN counts as a failure
    if bad.any():
        i = int(np.flatnonzero(bad)[np.argmax((err / np.maximum(scale, 1e-300))[bad])])
        raise AssertionError("%s: %d bins off; worst bin %d: gpu %.17g oracle %.17g scale %.3g "
                             "rel %.3g" % (what, int(bad.sum()), i, got[i], ref[i], scale[i],
                                           err[i] / max(scale[i], 1e-300)))
    return float(np.max(err / np.maximum(scale, 1e-300))) if len(err) else 0.0


# grids used by the parity tests
def make_grid(kind, n, rng):
    if kind == "geo_fine":        # x_i = 1e-21 2^(i/16): ties 2 x_j = x_{j+16} are exact
        return pg.grids.geometric_pow2(n, 1e-21, 16.0)
    if kind == "geo_ref":         # the reference tests' grid, by repeated multiplication
        return pg.grids.geometric_by_product(n, 1e-18, 1.122018)
    if kind == "geo_coarse":      # ratio 2: x_j + x_k lands exactly on pivots often
        return np.ldexp(1e-150, np.arange(n))             # exact, finite up to n ~ 1500
    if kind == "generic":         # non-geometric, strictly increasing, spans ~e^40
        steps = rng.uniform(0.2, 1.8, size=n) * (40.0 / max(n, 1))
        return 1e-20 * np.exp(np.cumsum(steps))
    if kind == "generic_wide":    # non-geometric, ~0.2 e-folds per bin (e^230 at n = 1111)
        steps = rng.uniform(0.02, 0.4, size=n)
        return 1e-20 * np.exp(np.cumsum(steps))
    if kind == "linear":          # x_i = (i+1) h: half the pairs are clipped at x[n-1]
        return 1e-18 * np.arange(1, n + 1, dtype=np.float64)
    raise ValueError(kind)


def make_N(kind, x, rng):
    n = len(x)
    if kind == "lognormal":
        return pg.grids.lognormal_ic(x, max(0, n // 4), 1.0, 1e14)
    if kind == "random":
        N = rng.lognormal(mean=20.0, sigma=3.0, size=n)
        N[rng.random(n) < 0.2] = 0.0
        return N
    raise ValueError(kind)


AGG_KERNELS = [  # (kernel, beta0, beta_br, beta_sh)
    (0, 1e-15, 0.0, 0.0),
    (1, 1e-3, 0.0, 0.0),
    (2, 1e12, 0.0, 0.0),
    (3, 0.0, 6.73e-18, 0.0),
    (4, 0.0, 0.0, 66.67),
    (5, 0.0, 6.73e-18, 66.67),
]
