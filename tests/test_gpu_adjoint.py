"""Checkpointed RK4 adjoint (pbe_rk4_tape_*) on the GPU.

Checked three ways: against the oracle's serial discrete adjoint (itself
pinned to finite differences in test_oracle_rk4_adjoint.py), against central
finite differences of the GPU forward (h = 1e-6 relative), and for
independence of the checkpoint interval (bitwise). The two-stage flocculation
workload (shear rate switching mid-run, power-law selection and daughter,
L = sum x^(2/3) N(T)) is run at full size. A torch.autograd.Function wraps the
tape here, in the test harness only."""
import json
import os

import numpy as np
import pytest

import pbe_gb300 as pg
import pyoracle
from gpu_util import t

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    return torch


def small_case(n=200, steps=12, switch=6):
    x = pg.grids.geometric_pow2(n, 1e-21, 16.0)
    N0 = pg.grids.lognormal_ic(x, n // 4, 1.0, 1e13)
    t_q, bw_q = pg.quadrature.power_law(2.0, 4)
    v_ref = float(x[n // 2])
    agg = [pg.AggregationParams(n=n, kernel_type=5, beta0=0.0, beta_br=6.73e-18, beta_sh=4 * G / 3)
           for G in (100.0, 20.0)]
    brk = [pg.BreakageParams(n=n, n_quad=len(t_q), selection=2, S0=5e-4 * f, v_ref=v_ref,
                             alpha=1.0 + 0.1 * f) for f in (1.0, 2.0)]
    step_set = np.array([0 if s < switch else 1 for s in range(steps)], dtype=np.int32)
    return x, N0, t_q, bw_q, agg, brk, step_set


def run_tape(x, N0, t_q, bw_q, agg, brk, step_set, dt, every, lam):
    torch = _torch()
    n, m = len(x), len(agg if agg is not None else brk)
    with pg.Rk4Tape(len(step_set), dt, every, agg, brk, step_set) as tape:
        N = t(N0)
        dx, dtq, dbw = t(x), t(t_q), t(bw_q)
        assert tape.forward(N, dx, dtq, dbw) == 0
        gN0 = t(np.zeros(n))
        ga, gb = t(np.zeros(3 * m)), t(np.zeros(4 * m))
        assert tape.backward(t(lam), gN0, ga, gb) == 0
        torch.cuda.synchronize()
        return (N.cpu().numpy(), gN0.cpu().numpy(), ga.cpu().numpy().reshape(m, 3),
                gb.cpu().numpy().reshape(m, 4))


def oracle_sets(agg, brk):
    A = np.array([[a.kernel_type, a.beta0, a.beta_br, a.beta_sh] for a in agg])
    B = np.array([[b.selection, b.S0, b.v_ref, b.alpha, b.v_min] for b in brk])
    return A, B


def test_tape_matches_oracle_adjoint():
    x, N0, t_q, bw_q, agg, brk, step_set = small_case()
    dt = 0.5
    lam = x ** (2.0 / 3.0)
    NT, gN0, ga, gb = run_tape(x, N0, t_q, bw_q, agg, brk, step_set, dt, 5, lam)
    A, B = oracle_sets(agg, brk)
    rNT, rgN0, rga, rgb = pyoracle.rk4_adjoint(N0, x, dt, len(step_set), lam, A, B, step_set,
                                               t_q, bw_q)
    np.testing.assert_allclose(NT, rNT, rtol=1e-11, atol=1e-11 * np.abs(N0).max())
    np.testing.assert_allclose(gN0, rgN0, rtol=1e-10, atol=1e-10 * np.abs(rgN0).max())
    np.testing.assert_allclose(ga[:, 1:], rga[:, 1:], rtol=1e-9)
    np.testing.assert_allclose(gb[:, [0, 2]], rgb[:, [0, 2]], rtol=1e-9)
    np.testing.assert_allclose(gb[:, 1], rgb[:, 1], rtol=1e-9, atol=1e-9 * np.abs(rgb[:, 1]).max())


@pytest.mark.parametrize("with_breakage", [False, True], ids=["agg", "agg+brk"])
def test_tape_forward_equals_drop_in_calls(with_breakage):
    """The tape keeps the grid-only tables per parameter set and recomputes
    only the N-dependent part of each RHS. Its RK4 steps are compared with RK4
    driven from the host through the drop-in calls (gather mode) with the
    reference examples' stage arithmetic (each product and sum rounded on its
    own), across a switch of parameter set: bit for bit for aggregation (the
    same kernels on cached tables); with breakage within 1e-14 relative per
    bin, because the drop-in breakage call gathers in one pass with the share
    factors regrouped while the tape gathers from its cached fragment
    brackets (a last-bit difference)."""
    torch = _torch()
    for n, q in ((3840, 128.0), (500, 16.0)):
        x = pg.grids.geometric_pow2(n, 1e-21, q)
        N0 = pg.grids.lognormal_ic(x, n // 6, 1.0, 1e12, cut=5.0)
        t_q, bw_q = pg.quadrature.power_law(2.0, 4)
        agg = [pg.AggregationParams(n=n, kernel_type=5, beta0=0.0, beta_br=6.73e-18,
                                    beta_sh=4 * G / 3) for G in (100.0, 20.0)]
        brk = [pg.BreakageParams(n=n, n_quad=len(t_q), selection=2, S0=5e-4 * f, v_ref=1e-18,
                                 alpha=1.0 + 0.2 * f) for f in (1.0, 2.0)]
        if not with_breakage:
            brk = None
        step_set = np.array([0, 0, 1, 1], dtype=np.int32)
        dt = 0.5
        dx, dtq, dbw = t(x), t(t_q), t(bw_q)
        with pg.Rk4Tape(len(step_set), dt, 2, agg, brk, step_set) as tape:
            Nt = t(N0)
            assert tape.forward(Nt, dx, dtq, dbw) == 0
            torch.cuda.synchronize()
        N = t(N0)

        def f(Y, m):
            k = torch.zeros(n, dtype=torch.float64, device="cuda")
            assert pg.aggregation_rhs(Y, dx, k, agg[m], mode=pg.MODE_GATHER) == 0
            if brk is not None:
                assert pg.breakage_rhs(Y, dx, dtq, dbw, k, brk[m], mode=pg.MODE_GATHER) == 0
            return k
        h, dt6 = 0.5 * dt, dt / 6.0
        for m in step_set:
            k1 = f(N, m)
            k2 = f(N + h * k1, m)
            k3 = f(N + h * k2, m)
            k4 = f(N + dt * k3, m)
            acc = k1 + 2.0 * k2
            acc = acc + 2.0 * k3
            N = N + dt6 * (acc + k4)
        torch.cuda.synchronize()
        a, b = Nt.cpu().numpy(), N.cpu().numpy()
        if with_breakage:
            np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(b).max())
        else:
            assert np.array_equal(a.view(np.int64), b.view(np.int64)), \
                "n=%d: %d bins differ, max rel %.3e" % (
                    n, int((a != b).sum()),
                    float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))))


def test_checkpoint_interval_does_not_change_the_result():
    x, N0, t_q, bw_q, agg, brk, step_set = small_case(n=120, steps=9, switch=4)
    lam = np.random.default_rng(3).normal(size=len(x))
    outs = [run_tape(x, N0, t_q, bw_q, agg, brk, step_set, 0.5, every, lam)
            for every in (1, 4, 9, 50)]
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_tape_matches_finite_differences_of_gpu_forward():
    torch = _torch()
    x, N0, t_q, bw_q, agg, brk, step_set = small_case(n=160, steps=8, switch=4)
    dt = 0.5
    w = x ** (2.0 / 3.0)
    _, gN0, ga, gb = run_tape(x, N0, t_q, bw_q, agg, brk, step_set, dt, 3, w)
    dx, dtq, dbw = t(x), t(t_q), t(bw_q)

    def L(N0_=N0, agg_=agg, brk_=brk):
        with pg.Rk4Tape(len(step_set), dt, 4, agg_, brk_, step_set) as tape:
            N = t(N0_)
            assert tape.forward(N, dx, dtq, dbw) == 0
            torch.cuda.synchronize()
            return float(w @ N.cpu().numpy())

    L0 = abs(L())
    for m in (10, 40, 41, 80, 120):
        h = 1e-6 * N0[m]
        Np, Nm = N0.copy(), N0.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (L(Np) - L(Nm)) / (2 * h)
        assert abs(fd - gN0[m]) <= 1e-6 * abs(gN0[m]) + 1e-12 * L0 / h, (m, fd, gN0[m])

    def perturbed(sets, k, name, h):
        out = []
        for i, s in enumerate(sets):
            c = type(s).from_buffer_copy(s)
            if i == k:
                setattr(c, name, getattr(c, name) + h)
            out.append(c)
        return out

    for k in range(2):
        for name, g in (("beta_br", ga[k, 1]), ("beta_sh", ga[k, 2])):
            h = 1e-6 * getattr(agg[k], name)
            fd = (L(agg_=perturbed(agg, k, name, h)) - L(agg_=perturbed(agg, k, name, -h))) / (2 * h)
            assert abs(fd - g) <= 2e-6 * abs(g) + 1e-12 * L0 / h, (k, name, fd, g)
        for name, g in (("S0", gb[k, 0]), ("alpha", gb[k, 2])):
            h = 1e-6 * getattr(brk[k], name)
            fd = (L(brk_=perturbed(brk, k, name, h)) - L(brk_=perturbed(brk, k, name, -h))) / (2 * h)
            assert abs(fd - g) <= 2e-6 * abs(g) + 1e-12 * L0 / h, (k, name, fd, g)


def test_autograd_function_wrapper():
    """The tape behind torch.autograd (harness-only wrapper): gradient of
    L = sum w N(T) with respect to N(0) equals the tape's dL/dN(0)."""
    torch = _torch()
    x, N0, t_q, bw_q, agg, brk, step_set = small_case(n=96, steps=6, switch=3)
    dt = 0.5
    dx, dtq, dbw = t(x), t(t_q), t(bw_q)

    class RK4Run(torch.autograd.Function):
        @staticmethod
        def forward(ctx, N0_):
            tape = pg.Rk4Tape(len(step_set), dt, 2, agg, brk, step_set)
            N = N0_.detach().clone().contiguous()
            assert tape.forward(N, dx, dtq, dbw) == 0
            ctx.tape = tape
            return N

        @staticmethod
        def backward(ctx, g):
            gN0 = torch.zeros_like(g)
            ga = torch.zeros(6, dtype=torch.float64, device=g.device)
            gb = torch.zeros(8, dtype=torch.float64, device=g.device)
            assert ctx.tape.backward(g.contiguous(), gN0, ga, gb) == 0
            ctx.tape.close()
            return gN0

    N0t = t(N0).requires_grad_(True)
    w = t(x ** (2.0 / 3.0))
    L = (w * RK4Run.apply(N0t)).sum()
    (g,) = torch.autograd.grad(L, N0t)
    _, gN0, _, _ = run_tape(x, N0, t_q, bw_q, agg, brk, step_set, dt, 2, x ** (2.0 / 3.0))
    assert np.array_equal(g.cpu().numpy(), gN0)


def test_flocculation_two_stage_adjoint_full_size():
    """n = 3840, 200 RK4 steps, checkpoints every 20, shear switching at step
    100: the forward equals the serial oracle's run of the same workload
    (committed golden), the gradient is finite and matches central differences
    for a few initial bins, the shear coefficient, the selection prefactor S0
    and the power-law exponent a of both stages."""
    torch = _torch()
    cfg = pg.grids.config_flocculation_adjoint()
    x, N0 = cfg["x"], cfg["N0"]
    agg, brk, ss = cfg["agg_sets"], cfg["brk_sets"], cfg["step_set"]
    NT, gN0, ga, gb = run_tape(x, N0, cfg["t_q"], cfg["bw_q"], agg, brk, ss, cfg["dt"], 20,
                               cfg["lam_T"])
    assert np.all(np.isfinite(NT)) and np.all(np.isfinite(gN0))
    assert np.all(np.isfinite(ga)) and np.all(np.isfinite(gb))
    # forward against the serial oracle's run of the same workload
    # (tests/golden/flocculation_two_stage.json, make_flocculation_golden.py)
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                       "flocculation_two_stage.json")))
    assert abs(float(cfg["lam_T"] @ NT) - gold["L"]) <= 1e-11 * abs(gold["L"])
    np.testing.assert_allclose(NT[::gold["every"]], gold["N_T"], rtol=1e-10,
                               atol=1e-10 * max(gold["N_T"]))
    dx, dtq, dbw = t(x), t(cfg["t_q"]), t(cfg["bw_q"])

    def L(N0_=N0, agg_=agg, brk_=brk):
        with pg.Rk4Tape(len(ss), cfg["dt"], 50, agg_, brk_, ss) as tape:
            N = t(N0_)
            assert tape.forward(N, dx, dtq, dbw) == 0
            torch.cuda.synchronize()
            return float(cfg["lam_T"] @ N.cpu().numpy())

    L0 = abs(L())
    for m in (400, 640, 900):
        h = 1e-6 * N0[m]
        Np, Nm = N0.copy(), N0.copy()
        Np[m] += h
        Nm[m] -= h
        fd = (L(Np) - L(Nm)) / (2 * h)
        assert abs(fd - gN0[m]) <= 1e-5 * abs(gN0[m]) + 1e-11 * L0 / h, (m, fd, gN0[m])
    for k in range(2):
        h = 1e-6 * agg[k].beta_sh
        ap = [type(a).from_buffer_copy(a) for a in agg]
        am = [type(a).from_buffer_copy(a) for a in agg]
        ap[k].beta_sh += h
        am[k].beta_sh -= h
        fd = (L(agg_=ap) - L(agg_=am)) / (2 * h)
        assert abs(fd - ga[k, 2]) <= 1e-5 * abs(ga[k, 2]) + 1e-11 * L0 / h, (k, fd, ga[k, 2])
    # selection prefactor S0 and power-law exponent a of both stages
    for k in range(2):
        for name, g in (("S0", gb[k, 0]), ("alpha", gb[k, 2])):
            h = 1e-6 * getattr(brk[k], name)
            bp = [type(b).from_buffer_copy(b) for b in brk]
            bm = [type(b).from_buffer_copy(b) for b in brk]
            setattr(bp[k], name, getattr(bp[k], name) + h)
            setattr(bm[k], name, getattr(bm[k], name) - h)
            fd = (L(brk_=bp) - L(brk_=bm)) / (2 * h)
            assert abs(fd - g) <= 1e-5 * abs(g) + 1e-11 * L0 / h, (k, name, fd, g)


def test_flocculation_adjoint_20_steps_matches_serial_oracle_adjoint():
    """The flocculation workload at full width (n = 3840) cut to 20 steps
    (shear switching at step 10), checkpoints every 5: every gradient the tape
    returns -- dL/dN(0), dL/dbeta_br, dL/dbeta_sh, dL/dS0 and dL/da of both
    stages -- against the serial FP64 discrete adjoint of the oracle (no
    checkpointing; tests/golden/flocculation_adjoint_20steps.npz, generator
    make_flocculation_adjoint_golden.py). Bounds as the small-case oracle
    comparison: rtol 1e-10 on dL/dN(0), 1e-9 on the coefficients."""
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden",
                                "flocculation_adjoint_20steps.npz"))
    steps, switch = int(gold["n_steps"]), int(gold["switch_step"])
    cfg = pg.grids.config_flocculation_adjoint(n_steps=steps, switch_step=switch)
    NT, gN0, ga, gb = run_tape(cfg["x"], cfg["N0"], cfg["t_q"], cfg["bw_q"], cfg["agg_sets"],
                               cfg["brk_sets"], cfg["step_set"], cfg["dt"], 5, cfg["lam_T"])
    np.testing.assert_allclose(NT, gold["N_T"], rtol=1e-11, atol=1e-11 * np.abs(cfg["N0"]).max())
    np.testing.assert_allclose(gN0, gold["gN0"], rtol=1e-10, atol=1e-10 * np.abs(gold["gN0"]).max())
    np.testing.assert_allclose(ga[:, 1:], gold["g_agg"][:, 1:], rtol=1e-9)       # beta_br, beta_sh
    np.testing.assert_allclose(gb[:, [0, 2]], gold["g_brk"][:, [0, 2]], rtol=1e-9)  # S0, a
    print("20-step adjoint vs oracle: max rel dL/dN0 %.2e, coefficients %s vs %s" % (
        float(np.max(np.abs(gN0 - gold["gN0"])) / np.abs(gold["gN0"]).max()),
        np.r_[ga[:, 1:].ravel(), gb[:, [0, 2]].ravel()].tolist(),
        np.r_[gold["g_agg"][:, 1:].ravel(), gold["g_brk"][:, [0, 2]].ravel()].tolist()))
