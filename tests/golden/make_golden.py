"""Generates tests/golden/golden_ref.npz: RHS vectors computed by the
reference's own CUDA kernels (acuoci/pbe-fixed-pivot-cuda src/aggregation.cu,
src/breakage.cu built unmodified by oracle/build_ref.sh, launched by
oracle/ref_runner.cpp with the reference launch geometry) on seeded inputs.

Run on a GPU machine from the repository root:
    python tests/golden/make_golden.py --out tests/golden/golden_ref.npz
The CPU test tests/test_oracle_golden.py checks the oracle against the file.
The reference accumulates with atomics, so its last bits depend on the
schedule; the check uses the per-bin bound |oracle - golden| <= 1e-12 * scale.
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for p in (os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300"), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)


def grids():
    rng = np.random.default_rng(2026)
    out = {}
    x = np.empty(64)
    x[0] = 1e-18
    for i in range(1, 64):
        x[i] = x[i - 1] * 1.122018
    out["ref64"] = (x, True)                                   # reference unit-test grid
    out["pow96"] = (1e-21 * np.power(2.0, np.arange(96) / 16.0), True)
    out["gen80"] = (1e-20 * np.exp(np.cumsum(rng.uniform(0.02, 0.4, 80))), False)
    return out


def populations(x, rng):
    n = len(x)
    N1 = 1e12 * np.exp(-np.arange(n) / 10.0)                  # reference conservation IC
    N2 = rng.lognormal(20.0, 3.0, n)
    N2[rng.random(n) < 0.2] = 0.0
    return {"exp": N1, "rand": N2}


AGG = [(0, 1e-15, 0.0, 0.0), (1, 1e-3, 0.0, 0.0), (2, 1e12, 0.0, 0.0), (3, 0.0, 6.73e-18, 0.0),
       (4, 0.0, 0.0, 66.67), (5, 0.0, 6.73e-18, 66.67)]


def daughters():
    from pbe_gb300 import quadrature as q

    return {"sym": q.symmetric_binary(), "ero": q.erosion(0.05), "uni8": q.uniform(8),
            "pow2": q.power_law(2.0, 4)}


def main():
    import torch

    import pbe_gb300 as pg
    import pyoracle

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    ref = pyoracle.RefRunner()
    rng = np.random.default_rng(7)
    f64 = dict(dtype=torch.float64, device="cuda")
    store = {}
    for gname, (x, geo) in grids().items():
        n = len(x)
        lx0, ilr = (math.log(x[0]), 1.0 / math.log(x[1] / x[0])) if geo else (0.0, 0.0)
        for pname, N in populations(x, rng).items():
            for k, b0, bbr, bsh in AGG:
                p = pg.AggregationParams(n=n, log_x0=lx0, inv_log_r=ilr, kernel_type=k, beta0=b0,
                                         beta_br=bbr, beta_sh=bsh)
                r = torch.zeros(n, **f64)
                assert ref.aggregation_rhs(torch.tensor(N, **f64), torch.tensor(x, **f64), r, p) == 0
                torch.cuda.synchronize()
                key = "agg/%s/%s/%d" % (gname, pname, k)
                store[key + "/x"] = x
                store[key + "/N"] = N
                store[key + "/params"] = np.array([n, lx0, ilr, k, b0, bbr, bsh])
                store[key + "/rhs"] = r.cpu().numpy()
            for dname, (t_q, bw_q) in daughters().items():
                for sel, S0, alpha in ((0, 1e-3, 1.0), (1, 1e-3, 1.0), (2, 5e-4, 1.5), (3, 1e-3, 1.0)):
                    vref = float(x[n // 2]) if sel in (1, 2) else 1.0
                    vmin = float(x[n // 2]) if sel == 3 else 0.0
                    p = pg.BreakageParams(n=n, n_quad=len(t_q), selection=sel, S0=S0, v_ref=vref,
                                          alpha=alpha, v_min=vmin)
                    r = torch.zeros(n, **f64)
                    assert ref.breakage_rhs(torch.tensor(N, **f64), torch.tensor(x, **f64),
                                            torch.tensor(t_q, **f64), torch.tensor(bw_q, **f64),
                                            r, p) == 0
                    torch.cuda.synchronize()
                    key = "brk/%s/%s/%s/%d" % (gname, pname, dname, sel)
                    store[key + "/x"] = x
                    store[key + "/N"] = N
                    store[key + "/t_q"] = t_q
                    store[key + "/bw_q"] = bw_q
                    store[key + "/params"] = np.array([n, len(t_q), sel, S0, vref, alpha, vmin])
                    store[key + "/rhs"] = r.cpu().numpy()
    np.savez_compressed(args.out, **store)
    print("wrote %d arrays to %s" % (len(store), args.out))


if __name__ == "__main__":
    main()
