"""GPU vector-Jacobian products vs the oracle's adjoint (itself pinned to
finite differences of the oracle forward in test_oracle_vjp.py), and vs
central finite differences of the GPU forward RHS.

Bound per entry: |gpu - oracle| <= 1e-12 * s + 1e-280, s = the oracle's sum of
|terms| for that entry (see oracle_aggregation_rhs_vjp)."""
import math

import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import AGG_KERNELS, agg_params, assert_close, make_N, make_grid, t

pytestmark = pytest.mark.gpu


def gpu_agg_vjp(N, x, lam, p):
    import torch

    gN = torch.zeros(len(x), dtype=torch.float64, device="cuda")
    gp = torch.zeros(3, dtype=torch.float64, device="cuda")
    code = pg.aggregation_rhs_vjp(t(N), t(x), t(lam), gN, gp, p)
    torch.cuda.synchronize()
    return code, gN.cpu().numpy(), gp.cpu().numpy()


def gpu_brk_vjp(N, x, t_q, bw_q, lam, p):
    import torch

    gN = torch.zeros(len(x), dtype=torch.float64, device="cuda")
    gp = torch.zeros(4, dtype=torch.float64, device="cuda")
    code = pg.breakage_rhs_vjp(t(N), t(x), t(t_q), t(bw_q), t(lam), gN, gp, p)
    torch.cuda.synchronize()
    return code, gN.cpu().numpy(), gp.cpu().numpy()


@pytest.mark.parametrize("grid", ["geo_fine", "geo_ref", "geo_coarse", "generic", "linear"])
@pytest.mark.parametrize("kernel,b0,bbr,bsh", AGG_KERNELS, ids=[str(k[0]) for k in AGG_KERNELS])
def test_aggregation_vjp_matches_oracle(kernel, b0, bbr, bsh, grid):
    rng = np.random.default_rng(500 + kernel)
    # 32, 33, 34, 65: around the lane path's row blocks of 32 (a last block
    # with one row and no lags, or with one lag)
    for n in (1, 2, 17, 32, 33, 34, 65, 300, 1000):
        if grid == "geo_coarse" and n > 700:
            continue   # x_n ~ 2^n: beta0 x_j x_k would overflow in the reference formula
        x = make_grid(grid, n, rng)
        N = make_N("random", x, rng)
        lam = rng.normal(size=n)
        p = agg_params(n, kernel, b0, bbr, bsh, x, geometric=grid.startswith("geo"))
        code, gN, gp = gpu_agg_vjp(N, x, lam, p)
        assert code == 0, pg.error_string(code)
        rN, rp, sN, sp, _ = pyoracle.aggregation_rhs_vjp(N, x, lam, kernel, b0, bbr, bsh, p.log_x0,
                                                         p.inv_log_r, exact_bracket=True,
                                                         with_scale=True)
        assert_close(gN, rN, sN, "dL/dN k=%d %s n=%d" % (kernel, grid, n))
        assert_close(gp, rp, sp, "dL/dbeta k=%d %s n=%d" % (kernel, grid, n))


DAUGHTERS = {"symmetric": pg.quadrature.symmetric_binary(), "erosion": pg.quadrature.erosion(0.05),
             "uniform8": pg.quadrature.uniform(8), "powerlaw2": pg.quadrature.power_law(2.0, 4)}


@pytest.mark.parametrize("daughter", list(DAUGHTERS))
@pytest.mark.parametrize("sel,S0,alpha", [(0, 1e-3, 1.0), (1, 1e-3, 1.0), (2, 5e-4, 1.5), (3, 1e-3, 1.0)])
def test_breakage_vjp_matches_oracle(sel, S0, alpha, daughter):
    rng = np.random.default_rng(900 + sel)
    t_q, bw_q = DAUGHTERS[daughter]
    for grid in ("geo_fine", "generic"):
        for n in (1, 3, 64, 1000):
            x = make_grid(grid, n, rng)
            N = make_N("random", x, rng)
            lam = rng.normal(size=n)
            mid = float(x[n // 2])
            p = pg.BreakageParams(n=n, n_quad=len(t_q), selection=sel, S0=S0, v_ref=mid,
                                  alpha=alpha, v_min=mid if sel == 3 else 0.0)
            code, gN, gp = gpu_brk_vjp(N, x, t_q, bw_q, lam, p)
            assert code == 0, pg.error_string(code)
            rN, rp, sN, sp, _ = pyoracle.breakage_rhs_vjp(N, x, t_q, bw_q, lam, sel, p.S0, p.v_ref,
                                                          p.alpha, p.v_min, with_scale=True)
            assert_close(gN, rN, sN, "brk dL/dN sel=%d %s n=%d" % (sel, grid, n))
            assert_close(gp, rp, sp, "brk dL/dparams sel=%d %s n=%d" % (sel, grid, n))


def test_vjp_is_bitwise_deterministic():
    rng = np.random.default_rng(2)
    n = 3000
    x = pg.grids.geometric_pow2(n, 1e-21, 256.0)
    N = pg.grids.lognormal_ic(x, 400, 1.0, 1e14)
    lam = rng.normal(size=n)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    outs = [gpu_agg_vjp(N, x, lam, p) for _ in range(3)]
    for o in outs[1:]:
        assert np.array_equal(o[1].view(np.int64), outs[0][1].view(np.int64))
        assert np.array_equal(o[2].view(np.int64), outs[0][2].view(np.int64))


def test_vjp_matches_finite_differences_of_gpu_forward():
    """dL/dN_m and dL/dbeta from central differences of L = lambda . rhs(N) with
    the GPU forward (gather mode), h = 1e-6 relative, at n = 2000."""
    import torch

    rng = np.random.default_rng(4)
    n = 2000
    x = pg.grids.geometric_pow2(n, 1e-21, 128.0)
    N = pg.grids.lognormal_ic(x, 300, 1.0, 1e14)
    lam = rng.normal(size=n)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    tx, tl = t(x), t(lam)

    def L(Nv, pp=p):
        rhs = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert pg.aggregation_rhs(t(Nv), tx, rhs, pp, mode=pg.MODE_GATHER) == 0
        return float(torch.dot(tl, rhs))

    _, gN, gp = gpu_agg_vjp(N, x, lam, p)
    Labs = abs(L(N)) + 1.0
    for m in (5, 250, 300, 310, 900, 1999):
        h = 1e-6 * N[m]
        Np, Nm = N.copy(), N.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (L(Np) - L(Nm)) / (2 * h)
        assert abs(fd - gN[m]) <= 1e-6 * abs(gN[m]) + 1e-9 * Labs / h, (m, fd, gN[m])
    for idx, name in ((1, "beta_br"), (2, "beta_sh")):
        base = getattr(p, name)
        hp = 1e-6 * base
        pp = agg_params(n, 5, 0.0, p.beta_br, p.beta_sh, x)
        pm = agg_params(n, 5, 0.0, p.beta_br, p.beta_sh, x)
        setattr(pp, name, base + hp)
        setattr(pm, name, base - hp)
        fd = (L(N, pp) - L(N, pm)) / (2 * hp)
        assert abs(fd - gp[idx]) <= 1e-6 * abs(gp[idx]) + 1e-9 * Labs / hp, (name, fd, gp[idx])


@pytest.mark.parametrize("kernel,b0,bbr,bsh", AGG_KERNELS, ids=[str(k[0]) for k in AGG_KERNELS])
def test_aggregation_vjp_matches_oracle_many_lag_chunks(kernel, b0, bbr, bsh):
    """n = 4500 on a geometric grid: the lane-block path with 18 lag chunks
    of 256 lags, 141 row blocks (the last one partial), rows whose larger-member
    sums come from two chunks of a block."""
    rng = np.random.default_rng(700 + kernel)
    n = 4500
    x = pg.grids.geometric_pow2(n, 1e-21, 256.0)
    N = make_N("random", x, rng)
    lam = rng.normal(size=n)
    p = agg_params(n, kernel, b0, bbr, bsh, x)
    code, gN, gp = gpu_agg_vjp(N, x, lam, p)
    assert code == 0, pg.error_string(code)
    rN, rp, sN, sp, _ = pyoracle.aggregation_rhs_vjp(N, x, lam, kernel, b0, bbr, bsh, p.log_x0,
                                                     p.inv_log_r, exact_bracket=True,
                                                     with_scale=True)
    assert_close(gN, rN, sN, "dL/dN k=%d n=%d" % (kernel, n))
    assert_close(gp, rp, sp, "dL/dbeta k=%d n=%d" % (kernel, n))


def test_aggregation_vjp_lane_and_tile_paths_agree_at_16384():
    """The bench's n = 16384 Brownian + shear case through the lane-block path
    (this process) and the row-tile path (a child process with
    PBE_GB300_VJP_PATH=tile): the same sums in another order, so within
    1e-12 of each entry's scale (the sum of |terms|, from the oracle at this
    size)."""
    import os
    import subprocess
    import sys
    import tempfile

    n = 16384
    x = pg.grids.geometric_pow2(n, 1e-21, 512.0)
    N = pg.grids.lognormal_ic(x, 2048, 1.0, 1e14)
    lam = np.random.default_rng(11).normal(size=n)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    code, gN, gp = gpu_agg_vjp(N, x, lam, p)
    assert code == 0
    here = os.path.dirname(os.path.abspath(__file__))
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "in.npz")
        dst = os.path.join(d, "out.npz")
        np.savez(src, N=N, x=x, lam=lam, log_x0=p.log_x0, inv_log_r=p.inv_log_r)
        child = (
            "import sys; sys.path[:0] = [%r, %r, %r]\n"
            "import numpy as np, torch, pbe_gb300 as pg\n"
            "from gpu_util import agg_params, t\n"
            "z = np.load(%r)\n"
            "n = len(z['x'])\n"
            "p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, z['x'])\n"
            "gN = torch.zeros(n, dtype=torch.float64, device='cuda')\n"
            "gp = torch.zeros(3, dtype=torch.float64, device='cuda')\n"
            "assert pg.aggregation_rhs_vjp(t(z['N']), t(z['x']), t(z['lam']), gN, gp, p) == 0\n"
            "np.savez(%r, gN=gN.cpu().numpy(), gp=gp.cpu().numpy())\n"
            % (here, os.path.join(os.path.dirname(here), "pbe-fixed-pivot-cuda_gb300"),
               os.path.join(os.path.dirname(here), "oracle"), src, dst))
        env = dict(os.environ, PBE_GB300_VJP_PATH="tile")
        subprocess.run([sys.executable, "-c", child], env=env, check=True, timeout=600)
        o = np.load(dst)
        tN, tp = o["gN"], o["gp"]
    rN, rp, sN, sp, _ = pyoracle.aggregation_rhs_vjp(N, x, lam, 5, 0.0, 6.73e-18, 66.67, p.log_x0,
                                                     p.inv_log_r, exact_bracket=True,
                                                     with_scale=True)
    assert_close(gN, tN, sN, "lane vs tile dL/dN")
    assert_close(gp, tp, sp, "lane vs tile dL/dbeta")
    assert_close(gN, rN, sN, "lane vs oracle dL/dN")
    assert_close(gp, rp, sp, "lane vs oracle dL/dbeta")
