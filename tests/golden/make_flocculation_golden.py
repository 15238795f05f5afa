"""Generates flocculation_two_stage.json: the oracle's forward result for the
two-stage flocculation adjoint workload (pbe_gb300.grids.
config_flocculation_adjoint: n = 3840, 200 RK4 steps, shear switching at step
100), i.e. L = sum x^(2/3) N(T), M0 and M1 of N(T) and every 64th bin of N(T).
Serial C++ oracle (oracle/pbe_oracle.cpp, oracle_rk4_step), about 10 minutes.

    python tests/golden/make_flocculation_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300"), os.path.join(ROOT, "oracle")]

import pbe_gb300 as pg  # noqa: E402
import pyoracle  # noqa: E402


def main():
    cfg = pg.grids.config_flocculation_adjoint()
    x, N = cfg["x"], cfg["N0"].copy()
    b = cfg["brk_sets"][0]
    for s in range(cfg["n_steps"]):
        a = cfg["agg_sets"][cfg["step_set"][s]]
        N = pyoracle.rk4_step(N, x, cfg["dt"],
                              agg=dict(kernel=5, beta0=0.0, beta_br=a.beta_br, beta_sh=a.beta_sh),
                              brk=dict(t_q=cfg["t_q"], bw_q=cfg["bw_q"], selection=2, S0=b.S0,
                                       v_ref=b.v_ref, alpha=b.alpha, v_min=0.0))
    out = {"what": "oracle forward of config_flocculation_adjoint (n=3840, 200 RK4 steps)",
           "L": float(cfg["lam_T"] @ N), "M0": float(N.sum()), "M1": float(x @ N),
           "every": 64, "N_T": [float(v) for v in N[::64]]}
    with open(os.path.join(HERE, "flocculation_two_stage.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(out["L"], out["M0"], out["M1"])


if __name__ == "__main__":
    main()
