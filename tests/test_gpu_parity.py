"""GPU library vs the CPU oracle, bin by bin (|gpu - oracle| <= 1e-12 * scale),
over every aggregation kernel and selection function, both accumulation modes,
geometric / generic / linear grids, tiny to mid sizes, plus the API contract
(rhs is added to, streams are honoured) and gather-mode determinism."""
import numpy as np
import pytest

import pbe_gb300 as pg
from gpu_util import (AGG_KERNELS, agg_params, assert_close, gpu_agg, gpu_brk, make_N, make_grid,
                      oracle_agg, oracle_brk, t)

pytestmark = pytest.mark.gpu

MODES = [pg.MODE_GATHER, pg.MODE_SCATTER]
GRIDS = ["geo_fine", "geo_ref", "geo_coarse", "generic", "generic_wide", "linear"]


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("kernel,b0,bbr,bsh", AGG_KERNELS, ids=[str(k[0]) for k in AGG_KERNELS])
def test_aggregation_matches_oracle(kernel, b0, bbr, bsh, grid, mode):
    rng = np.random.default_rng(1000 * kernel + len(grid))
    for n in (1, 2, 3, 17, 64, 300, 1111):
        if grid == "geo_coarse" and n > 700:
            continue   # x_n ~ 2^n: beta0 x_j x_k would overflow in the reference formula
        x = make_grid(grid, n, rng)
        for ic in ("lognormal", "random"):
            N = make_N(ic, x, rng)
            p = agg_params(n, kernel, b0, bbr, bsh, x, geometric=grid.startswith("geo"))
            code, got = gpu_agg(N, x, p, mode)
            assert code == 0, pg.error_string(code)
            ref, scale, _ = oracle_agg(N, x, p)
            assert_close(got, ref, scale, "k=%d grid=%s n=%d ic=%s" % (kernel, grid, n, ic))


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
@pytest.mark.parametrize("case", ["subnormal", "tiny", "wide"])
@pytest.mark.parametrize("kernel,b0,bbr,bsh", AGG_KERNELS, ids=[str(k[0]) for k in AGG_KERNELS])
def test_aggregation_product_scope_edges(kernel, b0, bbr, bsh, case, mode):
    """Number densities at the edges of the double range: a subnormal N, N so
    small that beta N underflows, and N spread over ~180 decades."""
    rng = np.random.default_rng(31 + kernel)
    for n in (40, 300):
        x = make_grid("geo_fine", n, rng)
        N = make_N("random", x, rng)
        if case == "subnormal":
            N[rng.integers(0, n, 3)] = 3e-310
        elif case == "tiny":
            N[rng.integers(0, n, 5)] = 1e-290          # beta * N underflows for small beta
        else:
            N *= np.exp(rng.uniform(-300.0, 120.0, size=n))
        p = agg_params(n, kernel, b0, bbr, bsh, x, geometric=True)
        code, got = gpu_agg(N, x, p, mode)
        assert code == 0, pg.error_string(code)
        ref, scale, _ = oracle_agg(N, x, p)
        assert_close(got, ref, scale, "k=%d case=%s n=%d" % (kernel, case, n))


DAUGHTERS = {
    "symmetric": pg.quadrature.symmetric_binary(),
    "symmetric16": pg.quadrature.symmetric_binary_split(16),
    "erosion": pg.quadrature.erosion(0.05),
    "uniform8": pg.quadrature.uniform(8),
    "powerlaw2": pg.quadrature.power_law(2.0, 4),
}
SELECTIONS = [  # (selection, S0, v_ref bin, alpha, v_min bin)
    (0, 1e-3, None, 1.0, None),
    (1, 1e-3, "mid", 1.0, None),
    (2, 5e-4, "mid", 1.5, None),
    (3, 1e-3, None, 1.0, "mid"),
]


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
@pytest.mark.parametrize("grid", ["geo_fine", "geo_ref", "generic"])
@pytest.mark.parametrize("daughter", list(DAUGHTERS))
@pytest.mark.parametrize("sel,S0,vref,alpha,vmin", SELECTIONS, ids=["const", "lin", "pow", "thr"])
def test_breakage_matches_oracle(sel, S0, vref, alpha, vmin, daughter, grid, mode):
    rng = np.random.default_rng(77 + sel)
    t_q, bw_q = DAUGHTERS[daughter]
    # 31, 32, 33, 62, 63: around the gather kernel's blocks (bin 0 alone, then 31 bins each)
    for n in (1, 2, 5, 31, 32, 33, 62, 63, 64, 1000):
        x = make_grid(grid, n, rng)
        N = make_N("random", x, rng)
        N[rng.random(n) < 0.05] = 1e-310    # below the 2.2e-308 guard
        mid = float(x[n // 2])
        p = pg.BreakageParams(n=n, n_quad=len(t_q), selection=sel, S0=S0,
                              v_ref=mid if vref else 1.0, alpha=alpha, v_min=mid if vmin else 0.0)
        code, got = gpu_brk(N, x, t_q, bw_q, p, mode)
        assert code == 0, pg.error_string(code)
        ref, scale, _ = oracle_brk(N, x, t_q, bw_q, p)
        assert_close(got, ref, scale, "sel=%d %s grid=%s n=%d" % (sel, daughter, grid, n))


@pytest.mark.parametrize("grid", ["geo_fine", "generic"])
@pytest.mark.parametrize("sel", [0, 2])
def test_breakage_gather_many_points(sel, grid):
    """136 quadrature points: in the gather kernel each warp takes 34 points and
    block 0's threads more than one point each (the prefix over the parents at
    or below x[0] and its per-point lookups)."""
    rng = np.random.default_rng(91 + sel)
    t_q, bw_q = pg.quadrature.uniform(136)
    for n in (3, 200, 2000):
        x = make_grid(grid, n, rng)
        N = make_N("random", x, rng)
        mid = float(x[n // 2])
        p = pg.BreakageParams(n=n, n_quad=len(t_q), selection=sel, S0=1e-3, v_ref=mid, alpha=1.5)
        code, got = gpu_brk(N, x, t_q, bw_q, p, pg.MODE_GATHER)
        assert code == 0, pg.error_string(code)
        ref, scale, _ = oracle_brk(N, x, t_q, bw_q, p)
        assert_close(got, ref, scale, "sel=%d grid=%s n=%d n_quad=136" % (sel, grid, n))


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
def test_calls_accumulate_into_rhs(mode):
    """rhs is added to (aggregation and breakage sharing one rhs), never overwritten."""
    rng = np.random.default_rng(5)
    n = 500
    x = make_grid("geo_fine", n, rng)
    N = make_N("lognormal", x, rng)
    prefill = rng.normal(size=n) * 1e3
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    code, got = gpu_agg(N, x, p, mode, rhs0=prefill)
    assert code == 0
    ref, scale, _ = oracle_agg(N, x, p)
    assert_close(got, ref + prefill, scale + np.abs(prefill), "prefilled rhs")
    t_q, bw_q = pg.quadrature.uniform(8)
    bp = pg.BreakageParams(n=n, n_quad=8, selection=2, S0=1e-3, v_ref=float(x[250]), alpha=1.0)
    code, got2 = gpu_brk(N, x, t_q, bw_q, bp, mode, rhs0=got)
    assert code == 0
    ref2, scale2, _ = oracle_brk(N, x, t_q, bw_q, bp)
    assert_close(got2, ref + prefill + ref2, scale + np.abs(prefill) + scale2, "agg+brk")


def test_side_stream_and_workspace():
    import torch

    rng = np.random.default_rng(9)
    n = 2000
    x = make_grid("geo_fine", n, rng)
    N = make_N("lognormal", x, rng)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    s = torch.cuda.Stream()
    tN, tx = t(N), t(x)
    rhs = torch.zeros(n, dtype=torch.float64, device="cuda")
    ws = torch.empty(pg.aggregation_workspace_bytes(n) // 8 + 32, dtype=torch.float64,
                     device="cuda")
    with torch.cuda.stream(s):
        code = pg.aggregation_rhs(tN, tx, rhs, p, stream=s, mode=pg.MODE_GATHER, workspace=ws)
    s.synchronize()
    assert code == 0
    ref, scale, _ = oracle_agg(N, x, p)
    assert_close(rhs.cpu().numpy(), ref, scale, "side stream + caller workspace")
    # too-small workspace is rejected
    small = torch.empty(16, dtype=torch.float64, device="cuda")
    assert pg.aggregation_rhs(tN, tx, rhs, p, mode=pg.MODE_GATHER, workspace=small) == \
        pg.ERR_INVALID_VALUE


def test_gather_mode_is_bitwise_deterministic():
    import torch

    rng = np.random.default_rng(11)
    n = 4096
    x = pg.grids.geometric_pow2(n, 1e-21, 512.0)
    N = pg.grids.lognormal_ic(x, 512, 1.0, 1e14)
    t_q, bw_q = pg.quadrature.uniform(16)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    bp = pg.BreakageParams(n=n, n_quad=16, selection=3, S0=1e-3, v_min=float(x[2048]))
    outs = []
    tN, tx, tt, tb = t(N), t(x), t(t_q), t(bw_q)
    for _ in range(4):
        rhs = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert pg.aggregation_rhs(tN, tx, rhs, p, mode=pg.MODE_GATHER) == 0
        assert pg.breakage_rhs(tN, tx, tt, tb, rhs, bp, mode=pg.MODE_GATHER) == 0
        outs.append(rhs.cpu().numpy().view(np.int64).copy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_volume_conservation_to_roundoff():
    """Interior aggregation and discrete daughters conserve sum x_i rhs_i to
    round-off: |sum x_i rhs_i| <= 1e-13 sum x_i scale_i (scale from the oracle).
    The population sits > 12 sigma away from both grid ends, so nothing is clipped."""
    n = 3000
    x = pg.grids.geometric_pow2(n, 1e-21, 128.0)
    N = pg.grids.lognormal_ic(x, 1500, 0.6, 1e14)
    t_q, bw_q = pg.quadrature.symmetric_binary()
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    bp = pg.BreakageParams(n=n, n_quad=1, selection=0, S0=1e-3)
    _, sa, _ = oracle_agg(N, x, p)
    _, sb, _ = oracle_brk(N, x, t_q, bw_q, bp)
    for mode in MODES:
        code, got = gpu_agg(N, x, p, mode)
        assert code == 0
        assert abs(np.sum(got * x)) <= 1e-13 * np.sum(sa * x)
        code, got = gpu_brk(N, x, t_q, bw_q, bp, mode)
        assert code == 0
        assert abs(np.sum(got * x)) <= 1e-13 * np.sum(sb * x)
