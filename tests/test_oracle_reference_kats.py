"""The oracle must satisfy every assertion of the reference's own unit tests
(tests/unit/test_aggregation.cpp, tests/unit/test_breakage.cpp), restated in
refsuite.py. CPU only."""
import numpy as np
import pytest

import pyoracle
import refsuite as rs


def _agg(N, x, p):
    if N is None:
        return 1, None   # the oracle has no pointers to null; the API rejects it
    rhs, _, code = pyoracle.aggregation_rhs(N, x, p["kernel_type"], p["beta0"], p["beta_br"],
                                            p["beta_sh"], p["log_x0"], p["inv_log_r"], n=p["n"])
    return code, rhs


def _brk(N, x, t_q, bw_q, p):
    if N is None:
        return 1, None
    rhs, _, code = pyoracle.breakage_rhs(N, x, t_q, bw_q, p["selection"], p["S0"], p["v_ref"],
                                         p["alpha"], p["v_min"], n=p["n"], n_quad=p["n_quad"])
    return code, rhs


@pytest.mark.parametrize("name,k,b0,bbr,bsh", rs.AGG_CASES)
def test_agg_smoke(name, k, b0, bbr, bsh):
    rs.agg_smoke(_agg, k, b0, bbr, bsh)


@pytest.mark.parametrize("name,k,b0,bbr,bsh", rs.AGG_CASES)
def test_agg_volume_conserved(name, k, b0, bbr, bsh):
    rs.agg_volume_conserved(_agg, k, b0, bbr, bsh)


def test_agg_zero_population():
    rs.agg_zero_population(_agg)


def test_agg_self_collision():
    rs.agg_self_collision(_agg)


def test_agg_total_number_nonincreasing():
    rs.agg_total_number_nonincreasing(_agg)


def test_agg_invalid_n():
    rs.agg_invalid_n(_agg)


@pytest.mark.parametrize("name,sel,kw", rs.BRK_SMOKE)
def test_brk_smoke(name, sel, kw):
    rs.brk_smoke(_brk, sel, kw)


@pytest.mark.parametrize("name,sel,kw", rs.BRK_SMOKE)
def test_brk_volume_conserved(name, sel, kw):
    rs.brk_volume_conserved(_brk, sel, kw)


def test_brk_zero_population():
    rs.brk_zero_population(_brk)


def test_brk_death_constant():
    rs.brk_death_constant(_brk)


def test_brk_total_number_nondecreasing():
    rs.brk_total_number_nondecreasing(_brk)


def test_brk_threshold_suppresses():
    rs.brk_threshold_suppresses(_brk)


def test_brk_invalid_n():
    rs.brk_invalid_n(_brk)


def test_oracle_rejects_bad_enums():
    x = rs.grid()
    N = np.ones(rs.N_BINS)
    assert pyoracle.aggregation_rhs(N, x, 6)[2] != 0
    assert pyoracle.breakage_rhs(N, x, rs.T_Q, rs.BW_Q, 4)[2] != 0


def test_oracle_rk4_constant_kernel_matches_scott():
    """Constant kernel, 1000 RK4 steps of dt = 1 s on x_i = 1e-18 2^i, n = 256:
    total number follows Smoluchowski/Scott M0(t) = M0(0) / (1 + beta0 M0(0) t / 2)
    independently of the initial distribution (pbe_examples_utils.hpp:207-221).
    The upper bins stay empty, so no mass is clipped."""
    n = 256
    x = 1e-18 * np.power(2.0, np.arange(n, dtype=np.float64))
    xm, N0, b0 = 4e-18, 1e12, 1e-15
    dx = x * np.sqrt(2.0) - x / np.sqrt(2.0)     # cell width on the geometric grid
    N = N0 * (x / xm) * np.exp(-x / xm) * dx / xm  # Delta x / x_m dimensionless
    M0 = N.sum()
    agg = dict(kernel=0, beta0=b0, log_x0=float(np.log(x[0])), inv_log_r=1.0 / np.log(2.0))
    for _ in range(1000):
        N = pyoracle.rk4_step(N, x, 1.0, agg=agg)
    expect = M0 / (1.0 + b0 * M0 * 1000.0 / 2.0)
    assert abs(N.sum() - expect) / expect < 1e-9
