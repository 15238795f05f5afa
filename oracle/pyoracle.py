"""ctypes binding of the CPU oracle and of the reference-kernel runner.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py (CPU-baseline leg and reference arm). The library never imports it.

  * liboracle.so (oracle/pbe_oracle.cpp): serial FP64 restatement of the
    reference RHS; returns rhs and the per-bin scale sum |contribution|.
  * libref_runner.so (oracle/ref_runner.cpp): launches the reference's own
    kernels from oracle/_ref/*.cubin (built by oracle/build_ref.sh).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
RUNNER_LIB = os.path.join(HERE, "_build", "libref_runner.so")
REF_AGG_CUBIN = os.path.join(HERE, "_ref", "ref_aggregation.cubin")
REF_BRK_CUBIN = os.path.join(HERE, "_ref", "ref_breakage.cubin")

_D = ctypes.POINTER(ctypes.c_double)
_o = None


def _lib():
    global _o
    if _o is None:
        if not os.path.isfile(ORACLE_LIB):
            raise ImportError("oracle not built: %s (run build())" % ORACLE_LIB)
        lib = ctypes.CDLL(ORACLE_LIB)
        lib.oracle_aggregation_rhs.restype = ctypes.c_int
        lib.oracle_aggregation_rhs.argtypes = [_D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_int]
        lib.oracle_aggregation_rhs_mt.restype = ctypes.c_int
        lib.oracle_aggregation_rhs_mt.argtypes = [_D, _D, _D, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, ctypes.c_int]
        lib.oracle_breakage_rhs.restype = ctypes.c_int
        lib.oracle_breakage_rhs.argtypes = [_D, _D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double]
        lib.oracle_aggregation_rhs_vjp.restype = ctypes.c_int
        lib.oracle_aggregation_rhs_vjp.argtypes = [_D, _D, _D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_int]
        lib.oracle_breakage_rhs_vjp.restype = ctypes.c_int
        lib.oracle_breakage_rhs_vjp.argtypes = [_D, _D, _D, _D, _D, _D, _D, _D, _D, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.oracle_aggregation_rhs_jvp.restype = ctypes.c_int
        lib.oracle_aggregation_rhs_jvp.argtypes = [_D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.oracle_breakage_rhs_jvp.restype = ctypes.c_int
        lib.oracle_breakage_rhs_jvp.argtypes = [_D, _D, _D, _D, _D, _D, _D, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.oracle_rk4_adjoint.restype = ctypes.c_int
        lib.oracle_rk4_adjoint.argtypes = [_D, _D, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int), ctypes.c_int, _D, _D, _D,
                                           _D, ctypes.c_int, _D, _D, _D, _D, _D]
        lib.oracle_rk4_step.restype = ctypes.c_int
        lib.oracle_rk4_step.argtypes = [_D, _D, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _D, _D, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double]
        _o = lib
    return _o


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def aggregation_rhs(N, x, kernel, beta0=1.0, beta_br=0.0, beta_sh=0.0, log_x0=0.0,
                    inv_log_r=0.0, rhs=None, n=None, exact_bracket=False,
                    with_misplaced=False):
    """Returns (rhs, scale, code) -- or (rhs, scale, misplaced, code) with
    with_misplaced -- accumulated into a copy of `rhs` (zeros if None).

    exact_bracket=False restates the reference literally (logarithm bracket on
    geometric grids); True uses the exact bracket x[lo] <= v < x[lo+1]
    everywhere. `misplaced` is the per-bin size of the reference's near-tie
    bracket misplacements (see oracle/pbe_oracle.cpp)."""
    N = _f64(N)
    x = _f64(x)
    n = len(x) if n is None else n
    out = np.zeros(max(n, 1)) if rhs is None else _f64(rhs).copy()
    scale = np.zeros_like(out)
    mis = np.zeros_like(out)
    code = _lib().oracle_aggregation_rhs(_dp(N), _dp(x), _dp(out), _dp(scale), _dp(mis), int(n),
                                         float(log_x0), float(inv_log_r), int(kernel),
                                         float(beta0), float(beta_br), float(beta_sh),
                                         1 if exact_bracket else 0)
    if with_misplaced:
        return out, scale, mis, code
    return out, scale, code


def aggregation_rhs_mt(N, x, kernel, beta0=1.0, beta_br=0.0, beta_sh=0.0, log_x0=0.0,
                       inv_log_r=0.0, nthreads=0):
    N = _f64(N)
    x = _f64(x)
    out = np.zeros(len(x))
    code = _lib().oracle_aggregation_rhs_mt(_dp(N), _dp(x), _dp(out), len(x), float(log_x0),
                                            float(inv_log_r), int(kernel), float(beta0),
                                            float(beta_br), float(beta_sh), int(nthreads))
    return out, code


def breakage_rhs(N, x, t_q, bw_q, selection, S0=1.0, v_ref=1.0, alpha=1.0, v_min=0.0,
                 rhs=None, n=None, n_quad=None):
    N = _f64(N)
    x = _f64(x)
    t_q = _f64(t_q)
    bw_q = _f64(bw_q)
    n = len(x) if n is None else n
    nq = len(t_q) if n_quad is None else n_quad
    out = np.zeros(max(n, 1)) if rhs is None else _f64(rhs).copy()
    scale = np.zeros_like(out)
    code = _lib().oracle_breakage_rhs(_dp(N), _dp(x), _dp(t_q), _dp(bw_q), _dp(out), _dp(scale),
                                      int(n), int(nq), int(selection), float(S0), float(v_ref),
                                      float(alpha), float(v_min))
    return out, scale, code


def aggregation_rhs_vjp(N, x, lam, kernel, beta0=1.0, beta_br=0.0, beta_sh=0.0, log_x0=0.0,
                        inv_log_r=0.0, exact_bracket=True, with_scale=False):
    """(dL/dN, [dL/dbeta0, dL/dbeta_br, dL/dbeta_sh], code) for L = lam . rhs_agg(N);
    with_scale adds the per-entry absolute scales: (gN, gp, sN, sp, code)."""
    N, x, lam = _f64(N), _f64(x), _f64(lam)
    gN, sN = np.zeros(len(x)), np.zeros(len(x))
    gp, sp = np.zeros(3), np.zeros(3)
    code = _lib().oracle_aggregation_rhs_vjp(_dp(N), _dp(x), _dp(lam), _dp(gN), _dp(gp), _dp(sN),
                                             _dp(sp), len(x), float(log_x0), float(inv_log_r),
                                             int(kernel), float(beta0), float(beta_br),
                                             float(beta_sh), 1 if exact_bracket else 0)
    if with_scale:
        return gN, gp, sN, sp, code
    return gN, gp, code


def breakage_rhs_vjp(N, x, t_q, bw_q, lam, selection, S0=1.0, v_ref=1.0, alpha=1.0, v_min=0.0,
                     with_scale=False):
    """(dL/dN, [dL/dS0, dL/dv_ref, dL/dalpha, dL/dv_min], code) for L = lam . rhs_brk(N);
    with_scale adds the per-entry absolute scales: (gN, gp, sN, sp, code)."""
    N, x, lam = _f64(N), _f64(x), _f64(lam)
    t_q, bw_q = _f64(t_q), _f64(bw_q)
    gN, sN = np.zeros(len(x)), np.zeros(len(x))
    gp, sp = np.zeros(4), np.zeros(4)
    code = _lib().oracle_breakage_rhs_vjp(_dp(N), _dp(x), _dp(t_q), _dp(bw_q), _dp(lam), _dp(gN),
                                          _dp(gp), _dp(sN), _dp(sp), len(x), len(t_q),
                                          int(selection), float(S0), float(v_ref), float(alpha),
                                          float(v_min))
    if with_scale:
        return gN, gp, sN, sp, code
    return gN, gp, code


def aggregation_rhs_jvp(N, v, x, kernel, beta0=1.0, beta_br=0.0, beta_sh=0.0):
    """(J(N) v, per-bin scale sum |contribution|, code) of the aggregation RHS."""
    N, v, x = _f64(N), _f64(v), _f64(x)
    out, scale = np.zeros(len(x)), np.zeros(len(x))
    code = _lib().oracle_aggregation_rhs_jvp(_dp(N), _dp(v), _dp(x), _dp(out), _dp(scale), len(x),
                                             int(kernel), float(beta0), float(beta_br),
                                             float(beta_sh))
    return out, scale, code


def breakage_rhs_jvp(N, v, x, t_q, bw_q, selection, S0=1.0, v_ref=1.0, alpha=1.0, v_min=0.0):
    """(J(N) v, per-bin scale, code) of the breakage RHS (guard on N)."""
    N, v, x = _f64(N), _f64(v), _f64(x)
    t_q, bw_q = _f64(t_q), _f64(bw_q)
    out, scale = np.zeros(len(x)), np.zeros(len(x))
    code = _lib().oracle_breakage_rhs_jvp(_dp(N), _dp(v), _dp(x), _dp(t_q), _dp(bw_q), _dp(out),
                                          _dp(scale), len(x), len(t_q), int(selection), float(S0),
                                          float(v_ref), float(alpha), float(v_min))
    return out, scale, code


def _rhs(N, x, agg, brk):
    out = np.zeros(len(x))
    if agg:
        out = aggregation_rhs(N, x, agg["kernel"], agg.get("beta0", 1.0), agg.get("beta_br", 0.0),
                              agg.get("beta_sh", 0.0), rhs=out, exact_bracket=True)[0]
    if brk:
        out = breakage_rhs(N, x, brk["t_q"], brk["bw_q"], brk["selection"], brk.get("S0", 1.0),
                           brk.get("v_ref", 1.0), brk.get("alpha", 1.0), brk.get("v_min", 0.0),
                           rhs=out)[0]
    return out


def jacobian(N, x, agg=None, brk=None):
    """Dense J(N) = d rhs / dN (column k = J e_k from the Jacobian-vector products)."""
    n = len(x)
    J = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        col = np.zeros(n)
        if agg:
            col += aggregation_rhs_jvp(N, e, x, agg["kernel"], agg.get("beta0", 1.0),
                                       agg.get("beta_br", 0.0), agg.get("beta_sh", 0.0))[0]
        if brk:
            col += breakage_rhs_jvp(N, e, x, brk["t_q"], brk["bw_q"], brk["selection"],
                                    brk.get("S0", 1.0), brk.get("v_ref", 1.0),
                                    brk.get("alpha", 1.0), brk.get("v_min", 0.0))[0]
        J[:, k] = col
    return J


def ros2_step(N, x, dt, agg=None, brk=None):
    """One ROS2 step (gamma = 1 + 1/sqrt 2) with the dense Jacobian at N and
    direct solves: (I - gamma dt J) k1 = R(N); (I - gamma dt J) k2 = R(N + dt k1)
    - 2 k1; N + 3/2 dt k1 + 1/2 dt k2. agg / brk as for rk4_step."""
    N, x = _f64(N), _f64(x)
    g = 1.0 + 1.0 / np.sqrt(2.0)
    A = np.eye(len(x)) - g * dt * jacobian(N, x, agg, brk)
    k1 = np.linalg.solve(A, _rhs(N, x, agg, brk))
    k2 = np.linalg.solve(A, _rhs(N + dt * k1, x, agg, brk) - 2.0 * k1)
    return N + (1.5 * dt * k1 + 0.5 * dt * k2)


def ros2_adaptive(N, x, t_end, rtol, atol, dt0, agg=None, brk=None, max_attempts=100000):
    """ROS2 to t_end with the step control of pbe_batch_ros2_adaptive (dense
    solves): err = RMS(dt (k1 + k2) / 2 / (atol + rtol max(|N|, |N_new|))),
    accept when <= 1, dt *= clamp(0.9 err^-1/2, 0.2, 5) (<= 1 after a
    rejection), never past t_end. Returns (N, steps, rejects, status)."""
    N, x = _f64(N).copy(), _f64(x)
    g = 1.0 + 1.0 / np.sqrt(2.0)
    t, dt = 0.0, min(dt0, t_end)
    steps = rejects = 0
    for _ in range(max_attempts):
        A = np.eye(len(x)) - g * dt * jacobian(N, x, agg, brk)
        k1 = np.linalg.solve(A, _rhs(N, x, agg, brk))
        k2 = np.linalg.solve(A, _rhs(N + dt * k1, x, agg, brk) - 2.0 * k1)
        Nn = N + dt * (1.5 * k1 + 0.5 * k2)
        sc = atol + rtol * np.maximum(np.abs(N), np.abs(Nn))
        err = np.sqrt(np.mean((dt * (0.5 * (k1 + k2)) / sc) ** 2))
        finite = np.isfinite(err)
        accept = bool(finite and err <= 1.0)
        fac = 0.2 if not finite else (5.0 if err == 0.0 else min(5.0, max(0.2, 0.9 / np.sqrt(err))))
        if not accept:
            fac = min(fac, 1.0)
        if accept:
            t += dt
            N = Nn
            steps += 1
        else:
            rejects += 1
        rem = t_end - t
        nd = min(dt * fac, rem)
        if accept and rem <= 1e-12 * max(abs(t_end), 1.0):
            return N, steps, rejects, 1
        if nd <= 1e-14 * max(abs(t_end), 1.0):
            return N, steps, rejects, 2
        dt = nd
    return N, steps, rejects, 0


def rk4_step(N, x, dt, agg=None, brk=None):
    """One classical RK4 step; agg = dict(kernel, beta0, beta_br, beta_sh[, log_x0, inv_log_r]),
    brk = dict(t_q, bw_q, selection, S0, v_ref, alpha, v_min). Returns the new N."""
    N = _f64(N).copy()
    x = _f64(x)
    a = agg or {}
    b = brk or {}
    tq = _f64(b["t_q"]) if brk else None
    bw = _f64(b["bw_q"]) if brk else None
    code = _lib().oracle_rk4_step(
        _dp(N), _dp(x), len(x), float(dt), int(a.get("kernel", -1)) if agg else -1,
        float(a.get("log_x0", 0.0)), float(a.get("inv_log_r", 0.0)), float(a.get("beta0", 1.0)),
        float(a.get("beta_br", 0.0)), float(a.get("beta_sh", 0.0)), _dp(tq), _dp(bw),
        len(tq) if brk else 0, int(b.get("selection", 0)), float(b.get("S0", 1.0)),
        float(b.get("v_ref", 1.0)), float(b.get("alpha", 1.0)), float(b.get("v_min", 0.0)))
    if code:
        raise RuntimeError("oracle_rk4_step failed")
    return N


def rk4_adjoint(N0, x, dt, n_steps, lamT, agg_sets=None, brk_sets=None, step_set=None,
                t_q=None, bw_q=None):
    """Serial discrete adjoint of n_steps RK4 steps. agg_sets: rows
    (kernel, beta0, beta_br, beta_sh); brk_sets: rows (selection, S0, v_ref,
    alpha, v_min); step_set: parameter-set index per step (default all 0).
    Returns (N_T, dL/dN0, g_agg [sets, 3], g_brk [sets, 4]) for L with
    dL/dN(T) = lamT."""
    N0, x, lamT = _f64(N0), _f64(x), _f64(lamT)
    n = len(x)
    A = None if agg_sets is None else _f64(np.atleast_2d(agg_sets))
    B = None if brk_sets is None else _f64(np.atleast_2d(brk_sets))
    n_sets = (A if A is not None else B).shape[0]
    ss = None
    if step_set is not None:
        ss = np.ascontiguousarray(step_set, dtype=np.int32)
    tq = None if t_q is None else _f64(t_q)
    bw = None if bw_q is None else _f64(bw_q)
    NT, gN0 = np.zeros(n), np.zeros(n)
    ga, gb = np.zeros((n_sets, 3)), np.zeros((n_sets, 4))
    code = _lib().oracle_rk4_adjoint(
        _dp(N0), _dp(x), n, float(dt), int(n_steps),
        None if ss is None else ss.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n_sets,
        _dp(A), _dp(B), _dp(tq), _dp(bw), 0 if tq is None else len(tq), _dp(lamT), _dp(NT),
        _dp(gN0), _dp(ga), _dp(gb))
    if code:
        raise RuntimeError("oracle_rk4_adjoint failed")
    return NT, gN0, ga, gb


class RefRunner:
    """The reference's CUDA kernels (unmodified, from oracle/_ref) on the GPU."""

    def __init__(self):
        if not (os.path.isfile(RUNNER_LIB) and os.path.isfile(REF_AGG_CUBIN)
                and os.path.isfile(REF_BRK_CUBIN)):
            raise FileNotFoundError("reference runner or cubins missing under oracle/")
        import torch  # noqa: F401  (initialises the runtime's primary context)

        torch.cuda.init()
        torch.zeros(1, device="cuda")
        from pbe_gb300 import AggregationParams, BreakageParams

        self._AP, self._BP = AggregationParams, BreakageParams
        lib = ctypes.CDLL(RUNNER_LIB)
        lib.ref_init.restype = ctypes.c_int
        lib.ref_init.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        lib.ref_aggregation_rhs.restype = ctypes.c_int
        lib.ref_aggregation_rhs.argtypes = [ctypes.c_void_p] * 3 + [ctypes.POINTER(AggregationParams),
                                                                     ctypes.c_void_p]
        lib.ref_breakage_rhs.restype = ctypes.c_int
        lib.ref_breakage_rhs.argtypes = [ctypes.c_void_p] * 5 + [ctypes.POINTER(BreakageParams),
                                                                  ctypes.c_void_p]
        code = lib.ref_init(REF_AGG_CUBIN.encode(), REF_BRK_CUBIN.encode())
        if code:
            raise RuntimeError("ref_init failed: %d" % code)
        self.lib = lib

    @staticmethod
    def _stream(stream):
        import torch

        s = torch.cuda.current_stream() if stream is None else stream
        return s.cuda_stream or None

    def aggregation_rhs(self, N, x, rhs, params, stream=None):
        return self.lib.ref_aggregation_rhs(N.data_ptr(), x.data_ptr(), rhs.data_ptr(), params,
                                            self._stream(stream))

    def breakage_rhs(self, N, x, t_q, bw_q, rhs, params, stream=None):
        return self.lib.ref_breakage_rhs(N.data_ptr(), x.data_ptr(), t_q.data_ptr(),
                                         bw_q.data_ptr(), rhs.data_ptr(), params,
                                         self._stream(stream))
