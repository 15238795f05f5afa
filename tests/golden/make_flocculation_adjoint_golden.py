"""Generates flocculation_adjoint_20steps.npz: the oracle's serial discrete
RK4 adjoint (oracle/pbe_oracle.cpp via pyoracle.rk4_adjoint, every stage state
kept, no checkpointing) of the two-stage flocculation workload cut to 20 steps
(pbe_gb300.grids.config_flocculation_adjoint(n_steps=20, switch_step=10):
n = 3840, x_i = 1e-21 2^(i/128), G = 100 -> 20 1/s at step 10, power-law
selection and daughter, dt = 0.5 s, L = sum x^(2/3) N(T)).

Stored: N_T, dL/dN(0) (all bins), dL/d(beta0, beta_br, beta_sh) per stage
[2, 3], dL/d(S0, v_ref, alpha, v_min) per stage [2, 4], L. About 2-3 minutes
of serial CPU.

    python tests/golden/make_flocculation_adjoint_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300"), os.path.join(ROOT, "oracle")]

import pbe_gb300 as pg  # noqa: E402
import pyoracle  # noqa: E402

N_STEPS, SWITCH = 20, 10


def main():
    cfg = pg.grids.config_flocculation_adjoint(n_steps=N_STEPS, switch_step=SWITCH)
    A = np.array([[a.kernel_type, a.beta0, a.beta_br, a.beta_sh] for a in cfg["agg_sets"]])
    B = np.array([[b.selection, b.S0, b.v_ref, b.alpha, b.v_min] for b in cfg["brk_sets"]])
    NT, gN0, ga, gb = pyoracle.rk4_adjoint(cfg["N0"], cfg["x"], cfg["dt"], N_STEPS, cfg["lam_T"],
                                           A, B, cfg["step_set"], cfg["t_q"], cfg["bw_q"])
    np.savez_compressed(os.path.join(HERE, "flocculation_adjoint_20steps.npz"),
                        N_T=NT, gN0=gN0, g_agg=ga, g_brk=gb, L=float(cfg["lam_T"] @ NT),
                        n_steps=N_STEPS, switch_step=SWITCH)
    print("L", float(cfg["lam_T"] @ NT), "g_agg", ga.tolist(), "g_brk", gb.tolist())


if __name__ == "__main__":
    main()
