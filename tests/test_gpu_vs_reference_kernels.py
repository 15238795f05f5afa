"""GPU library vs the reference's own CUDA kernels (built unmodified from its
sources into oracle/_ref/ and launched with its launch geometry by
oracle/ref_runner.cpp), on the same device and inputs, up to the full
single-instance workload n = 16384 (Brownian+shear, threshold breakage).
Per-bin bound: |lib - ref| <= 1e-12 * scale + misplaced (+1e-280), with scale
and misplaced from the CPU oracle run the reference's way: `misplaced` is what
the reference's logarithm bracket moves near ties relative to the exact
bracket the library uses (zero on generic grids and away from ties)."""
import os

import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import (AGG_KERNELS, agg_params, assert_close, make_N, make_grid,
                      oracle_agg_reference, t)

pytestmark = pytest.mark.gpu

if not os.path.isfile(pyoracle.REF_AGG_CUBIN):
    pytest.skip("reference kernels not built (oracle/_ref)", allow_module_level=True)


@pytest.fixture(scope="module")
def ref():
    return pyoracle.RefRunner()


def _run_ref_agg(ref, N, x, p):
    import torch

    rhs = torch.zeros(len(x), dtype=torch.float64, device="cuda")
    assert ref.aggregation_rhs(t(N), t(x), rhs, p) == 0
    torch.cuda.synchronize()
    return rhs.cpu().numpy()


def _run_lib_agg(N, x, p, mode):
    import torch

    rhs = torch.zeros(len(x), dtype=torch.float64, device="cuda")
    assert pg.aggregation_rhs(t(N), t(x), rhs, p, mode=mode) == 0
    torch.cuda.synchronize()
    return rhs.cpu().numpy()


@pytest.mark.parametrize("grid", ["geo_fine", "geo_ref", "generic"])
@pytest.mark.parametrize("kernel,b0,bbr,bsh", AGG_KERNELS, ids=[str(k[0]) for k in AGG_KERNELS])
def test_aggregation_vs_reference_kernels(ref, kernel, b0, bbr, bsh, grid):
    rng = np.random.default_rng(kernel)
    for n in (2, 64, 777, 2048):
        x = make_grid(grid, n, rng)
        N = make_N("random", x, rng)
        p = agg_params(n, kernel, b0, bbr, bsh, x, geometric=grid.startswith("geo"))
        r = _run_ref_agg(ref, N, x, p)
        _, scale, mis = oracle_agg_reference(N, x, p)
        for mode in (pg.MODE_GATHER, pg.MODE_SCATTER):
            assert_close(_run_lib_agg(N, x, p, mode), r, scale,
                         "k=%d %s n=%d mode=%d" % (kernel, grid, n, mode), extra=mis)


def test_full_size_workload_vs_reference_kernels(ref):
    """n = 16384, x_i = 1e-21 2^(i/512), lognormal N (median bin 2048,
    sigma_ln 1, total 1e14), Brownian+shear (6.73e-18, 4*50/3) plus threshold
    breakage (S0 1e-3, v_min = x_8192, symmetric daughter as 16 entries)."""
    import torch

    c = pg.grids.config_n16384()
    n, x, N = c["n"], c["x"], c["N"]
    p = agg_params(n, 5, 0.0, c["beta_br"], c["beta_sh"], x)
    t_q, bw_q = pg.quadrature.symmetric_binary_split(16)
    bp = pg.BreakageParams(n=n, n_quad=16, selection=3, S0=c["S0"], v_min=c["v_min"])
    tN, tx, tt, tb = t(N), t(x), t(t_q), t(bw_q)
    r = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert ref.aggregation_rhs(tN, tx, r, p) == 0
    assert ref.breakage_rhs(tN, tx, tt, tb, r, bp) == 0
    torch.cuda.synchronize()
    r = r.cpu().numpy()
    # oracle scale (all host threads)
    _, sa, mis = oracle_agg_reference(N, x, p)
    _, sb, _ = pyoracle.breakage_rhs(N, x, t_q, bw_q, 3, c["S0"], 1.0, 1.0, c["v_min"])
    for mode in (pg.MODE_GATHER, pg.MODE_SCATTER):
        out = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert pg.aggregation_rhs(tN, tx, out, p, mode=mode) == 0
        assert pg.breakage_rhs(tN, tx, tt, tb, out, bp, mode=mode) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        worst = assert_close(got, r, sa + sb, "n=16384 mode=%d" % mode, extra=mis)
        # size of the near-tie allowance: how far the reference's logarithm
        # bracket moves bins relative to the exact bracket, and how many bins
        # would miss the plain 1e-12 * scale bound without it
        scale = sa + sb
        rel_mis = mis / np.maximum(scale, 1e-300)
        plain = np.abs(got - r) > 1e-12 * scale + 1e-280
        print("n=16384 mode %d: worst |lib-ref|/scale = %.3e; near-tie allowance: max "
              "misplaced/scale = %.3e over %d bins with misplaced > 0; bins beyond 1e-12*scale "
              "without it: %d of %d (worst %.3e)"
              % (mode, worst, float(rel_mis.max()), int((mis > 0).sum()), int(plain.sum()), n,
                 float((np.abs(got - r) / np.maximum(scale, 1e-300)).max())))
