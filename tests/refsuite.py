"""The assertions of the reference's unit tests, restated once and replayed
against any RHS implementation (the CPU oracle in test_oracle_reference_kats.py,
the GPU library in test_gpu_reference_suite.py).

Source: acuoci/pbe-fixed-pivot-cuda tests/unit/test_aggregation.cpp (17 tests)
and tests/unit/test_breakage.cpp (14 tests). Fixture: N = 64 pivots,
x_0 = 1e-18, x_i = x_{i-1} * 1.122018 (test_aggregation.cpp:48-81);
symmetric binary daughter t = 0.5, bw = 2 (test_breakage.cpp:50-59).

An implementation is a pair of callables
    agg(N, x, params_dict) -> (code, rhs)
    brk(N, x, t_q, bw_q, params_dict) -> (code, rhs)
with rhs zero-initialised before the call, like the fixture's run().
"""
from __future__ import annotations

import math

import numpy as np

N_BINS = 64
V_MIN = 1.0e-18
R = 1.122018

AGG_CASES = [  # (name, kernel, beta0, beta_br, beta_sh) -- test_aggregation.cpp:130-231
    ("Constant", 0, 1e-17, 0.0, 0.0),
    ("Sum", 1, 1e-17, 0.0, 0.0),
    ("Product", 2, 1e-17, 0.0, 0.0),
    ("Brownian", 3, 0.0, 1e-17, 0.0),
    ("Shear", 4, 0.0, 0.0, 1e-17),
    ("BrownianShear", 5, 0.0, 1e-17, 1e-17),
]


def grid():
    x = np.empty(N_BINS)
    x[0] = V_MIN
    for i in range(1, N_BINS):
        x[i] = x[i - 1] * R
    return x


def agg_params(kernel, b0=1e-17, b_br=0.0, b_sh=0.0, n=N_BINS):
    x = grid()
    return dict(n=n, log_x0=math.log(x[0]), inv_log_r=1.0 / math.log(x[1] / x[0]),
                kernel_type=kernel, beta0=b0, beta_br=b_br, beta_sh=b_sh, block_size=256)


def brk_params(sel, S0=1e-3, v_ref=1e-18, alpha=1.0, v_min=0.0, n=N_BINS):
    return dict(n=n, n_quad=1, selection=sel, S0=S0, v_ref=v_ref, alpha=alpha, v_min=v_min,
                block_size=256)


T_Q = np.array([0.5])
BW_Q = np.array([2.0])


# ---- aggregation ------------------------------------------------------------
def agg_smoke(agg, kernel, b0, b_br, b_sh):
    N = np.zeros(N_BINS)
    N[N_BINS // 2] = 1e14
    code, _ = agg(N, grid(), agg_params(kernel, b0, b_br, b_sh))
    assert code == 0


def agg_volume_conserved(agg, kernel, b0, b_br, b_sh):
    x = grid()
    N = 1e12 * np.exp(-np.arange(N_BINS) / 10.0)
    code, rhs = agg(N, x, agg_params(kernel, b0, b_br, b_sh))
    assert code == 0
    dM1 = float(np.sum(rhs * x))
    M1 = float(np.sum(N * x))
    assert abs(dM1) <= 1e-6 * abs(M1), (dM1, M1)


def agg_zero_population(agg):
    code, rhs = agg(np.zeros(N_BINS), grid(), agg_params(0))
    assert code == 0
    assert np.all(rhs == 0.0)


def agg_self_collision(agg):
    j, Nj, b0 = N_BINS // 2, 1e14, 1e-17
    N = np.zeros(N_BINS)
    N[j] = Nj
    code, rhs = agg(N, grid(), agg_params(0, b0))
    assert code == 0
    expected = -b0 * Nj * Nj
    assert abs(rhs[j] - expected) <= abs(expected) * 1e-10, (rhs[j], expected)


def agg_total_number_nonincreasing(agg):
    code, rhs = agg(np.full(N_BINS, 1e12), grid(), agg_params(0))
    assert code == 0
    assert float(np.sum(rhs)) <= 0.0


def agg_invalid_n(agg):
    p = agg_params(0)
    p["n"] = 0
    code, _ = agg(np.zeros(N_BINS), grid(), p)
    assert code != 0


def agg_null_pointer(agg):
    code, _ = agg(None, grid(), agg_params(0))
    assert code != 0


# ---- breakage ---------------------------------------------------------------
BRK_SMOKE = [  # (name, selection, kwargs) -- test_breakage.cpp:137-162, v_ref / v_min from the grid
    ("Constant", 0, {}),
    ("Linear", 1, {"v_ref": "x32"}),
    ("PowerLaw", 2, {"v_ref": "x32", "alpha": 2.0}),
    ("Threshold", 3, {"v_ref": 1.0, "alpha": 1.0, "v_min": "x16"}),
]


def _resolve(kw):
    x = grid()
    out = {}
    for k, v in kw.items():
        out[k] = float(x[int(v[1:])]) if isinstance(v, str) else v
    return out


def brk_smoke(brk, sel, kw):
    N = np.zeros(N_BINS)
    N[N_BINS // 2] = 1e14
    code, _ = brk(N, grid(), T_Q, BW_Q, brk_params(sel, **_resolve(kw)))
    assert code == 0


def brk_volume_conserved(brk, sel, kw):
    x = grid()
    N = 1e12 * np.exp(-np.arange(N_BINS) / 10.0)
    code, rhs = brk(N, x, T_Q, BW_Q, brk_params(sel, **_resolve(kw)))
    assert code == 0
    dM1 = float(np.sum(rhs * x))
    M1 = float(np.sum(N * x))
    assert abs(dM1) <= 1e-4 * abs(M1), (dM1, M1)


def brk_zero_population(brk):
    code, rhs = brk(np.zeros(N_BINS), grid(), T_Q, BW_Q, brk_params(0))
    assert code == 0
    assert np.all(rhs == 0.0)


def brk_death_constant(brk):
    j, Nj, S0 = N_BINS // 2, 1e14, 1e-3
    N = np.zeros(N_BINS)
    N[j] = Nj
    code, rhs = brk(N, grid(), T_Q, BW_Q, brk_params(0, S0))
    assert code == 0
    expected = -S0 * Nj
    assert abs(rhs[j] - expected) <= abs(expected) * 1e-10, (rhs[j], expected)


def brk_total_number_nondecreasing(brk):
    code, rhs = brk(np.full(N_BINS, 1e12), grid(), T_Q, BW_Q, brk_params(0))
    assert code == 0
    assert float(np.sum(rhs)) >= 0.0


def brk_threshold_suppresses(brk):
    x = grid()
    tb = N_BINS // 2
    code, rhs = brk(np.full(N_BINS, 1e12), x, T_Q, BW_Q,
                    brk_params(3, 1e-3, 1.0, 1.0, float(x[tb])))
    assert code == 0
    assert np.all(rhs[:tb] >= 0.0)


def brk_invalid_n(brk):
    p = brk_params(0)
    p["n"] = 0
    code, _ = brk(np.zeros(N_BINS), grid(), T_Q, BW_Q, p)
    assert code != 0


def brk_null_pointer(brk):
    code, _ = brk(None, grid(), T_Q, BW_Q, brk_params(0))
    assert code != 0
