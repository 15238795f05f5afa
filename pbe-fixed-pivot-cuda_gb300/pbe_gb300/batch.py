"""Batched cells: many independent PBE instances with uneven section counts,
evaluated by one persistent launch per RHS and integrated with RK4 steps
captured in one CUDA graph (C ABI pbe_batch_*, include/pbe_gb300.h).

The reference has no batched interface: its callers loop over cells and call
launch_aggregation_rhs / launch_breakage_rhs per cell and per RK4 stage, with
host round trips between stages (examples/common/pbe_examples_utils.hpp:409-456).
`BatchPlan.rk4_percell` runs that per-cell launch loop (without the host round
trips) on the single-instance kernels, as a baseline and a cross-check.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import BATCH_BRK_PREP, BATCH_BRK_TASKS, BATCH_RETUNE, BATCH_TUNE, PbeError
from .rhs import _ptr, _stream

PARAM_FIELDS = ("beta0", "beta_br", "beta_sh", "S0", "v_ref", "alpha", "v_min", "reserved")


def cell_params(n_cells: int, **values) -> np.ndarray:
    """Host array [n_cells, 8] of pbe_batch_cell_params_t rows. Each keyword
    (beta0, beta_br, beta_sh, S0, v_ref, alpha, v_min) is a scalar or an array
    of n_cells; unspecified fields take the reference's struct defaults
    (beta0 = S0 = v_ref = alpha = 1, the others 0)."""
    defaults = dict(beta0=1.0, beta_br=0.0, beta_sh=0.0, S0=1.0, v_ref=1.0, alpha=1.0, v_min=0.0)
    unknown = set(values) - set(defaults)
    if unknown:
        raise TypeError("unknown cell parameters: %s" % sorted(unknown))
    defaults.update(values)
    out = np.zeros((n_cells, 8))
    for i, name in enumerate(PARAM_FIELDS[:7]):
        out[:, i] = np.broadcast_to(np.asarray(defaults[name], dtype=np.float64), (n_cells,))
    return out


def shard_cells(cell_n: Sequence[int], rank: int, world: int) -> np.ndarray:
    """Indices of the cells rank `rank` of `world` owns when independent cells
    are spread over GPUs (one plan per GPU, no exchange between them): a
    contiguous range in cell order, cut where the running pair count
    n (n + 1) / 2 crosses k / world of the total, so every rank gets about
    the same pair work."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank %d outside world %d" % (rank, world))
    n = np.asarray(cell_n, dtype=np.float64)
    cost = np.cumsum(n * (n + 1) / 2)
    total = cost[-1] if len(cost) else 0.0
    cuts = [0] + [int(np.searchsorted(cost, total * k / world, side="left")) + 1
                  for k in range(1, world)] + [len(n)]
    cuts = np.minimum(np.maximum.accumulate(cuts), len(n))
    return np.arange(cuts[rank], cuts[rank + 1])


class BatchPlan:
    """A plan over `cell_n` cells; cell c uses the first cell_n[c] pivots of
    grids[cell_grid[c]]. kernel: AGG_* or -1 (no aggregation); selection:
    SEL_* or -1 (no breakage) with the daughter table (t_q, bw_q).
    tune / retune: time the tile group sizes per size class (cached);
    breakage_gather: "prep" or "tasks" forces where the breakage term is
    gathered (bitwise the same result; by default the plan picks by its
    cell count)."""

    def __init__(self, grids: Sequence[np.ndarray], cell_n: Sequence[int],
                 cell_grid: Sequence[int], kernel: int, selection: int = -1,
                 t_q: Optional[np.ndarray] = None, bw_q: Optional[np.ndarray] = None,
                 tune: bool = False, retune: bool = False, stream=None,
                 breakage_gather: Optional[str] = None):
        lib = _lib.load()
        grid_n = np.ascontiguousarray([len(g) for g in grids], dtype=np.int32)
        grid_x = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float64) for g in grids]))
        cn = np.ascontiguousarray(cell_n, dtype=np.int32)
        cg = np.ascontiguousarray(cell_grid, dtype=np.int32)
        nq = 0
        tq = bw = None
        if selection >= 0:
            tq = np.ascontiguousarray(t_q, dtype=np.float64)
            bw = np.ascontiguousarray(bw_q, dtype=np.float64)
            nq = len(tq)
        flags = (BATCH_TUNE if tune else 0) | (BATCH_RETUNE if retune else 0)
        if breakage_gather is not None:
            # "prep" or "tasks": where the breakage term is gathered (the plan
            # picks by its cell count when None)
            flags |= {"prep": BATCH_BRK_PREP, "tasks": BATCH_BRK_TASKS}[breakage_gather]
        h = ctypes.c_void_p()
        code = lib.pbe_batch_create(
            ctypes.byref(h), len(grid_n), grid_n.ctypes.data, grid_x.ctypes.data, len(cn),
            cn.ctypes.data, cg.ctypes.data, int(kernel), int(selection), nq,
            None if tq is None else tq.ctypes.data, None if bw is None else bw.ctypes.data,
            flags, _stream(stream))
        if code:
            raise PbeError(code, "pbe_batch_create")
        self._h = h
        self.n_cells = len(cn)
        self.cell_n = cn.copy()
        self.offsets = np.zeros(self.n_cells + 1, dtype=np.int64)
        _lib.check(lib.pbe_batch_offsets(h, self.offsets.ctypes.data), "pbe_batch_offsets")
        self.total = int(self.offsets[-1])

    # -- calls ------------------------------------------------------------------
    def rhs(self, N, rhs, params, stream=None) -> int:
        """rhs += RHS(N) for every cell. N, rhs: packed float64 device arrays;
        params: device array [n_cells, 8] (cell_params layout)."""
        return _lib.load().pbe_batch_rhs(self._h, _ptr(N, "N"), _ptr(rhs, "rhs"),
                                         _ptr(params, "params"), _stream(stream))

    def rk4(self, N, params, dt: float, n_steps: int, stream=None) -> int:
        """n_steps RK4 steps in place on N, as one CUDA graph launch."""
        return _lib.load().pbe_batch_rk4(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                         float(dt), int(n_steps), _stream(stream))

    def rk4_prepare(self, N, params, dt: float, n_steps: int) -> int:
        """Capture the graph rk4() would launch, without running it."""
        return _lib.load().pbe_batch_rk4_prepare(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                                 float(dt), int(n_steps))

    def rk45(self, N, params, t_end: float, rtol: float = 1e-8, atol: float = 0.0,
             dt0: float = 1e-3, max_attempts: int = 100000, stream=None):
        """Adaptive Dormand-Prince 5(4) to t_end, a step size per cell.
        Returns (code, accepted steps per cell, rejected steps per cell, attempts);
        code 600 (ERR_NOT_READY) if max_attempts ran out."""
        steps = np.zeros(self.n_cells, dtype=np.int32)
        rejects = np.zeros(self.n_cells, dtype=np.int32)
        att = ctypes.c_int()
        code = _lib.load().pbe_batch_rk45(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                          float(t_end), float(rtol), float(atol), float(dt0),
                                          int(max_attempts), steps.ctypes.data, rejects.ctypes.data,
                                          ctypes.byref(att), _stream(stream))
        return code, steps, rejects, att.value

    def rk4_percell(self, N, params, dt: float, n_steps: int, stream=None) -> int:
        """The same integration as a per-cell launch loop (baseline)."""
        return _lib.load().pbe_batch_rk4_percell(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                                 float(dt), int(n_steps), _stream(stream))

    def death(self, N, death, params, method: int = _lib.DEATH_MOMENTS, stream=None) -> int:
        """death[off_c + i] = N_ci sum_k beta_c(x_i, x_k) N_ck (overwritten), by the
        per-cell moments (DEATH_MOMENTS) or the FP64 tensor-core GEMM (DEATH_DMMA)."""
        return _lib.load().pbe_batch_death(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                           _ptr(death, "death"), int(method), _stream(stream))

    def rhs_vjp(self, N, lam, gN, gparams, params, stream=None) -> int:
        """gN += dL/dN, gparams[c, j] += dL/d(parameter j of cell c) for
        L = lam . RHS(N); gparams: device array [n_cells, 8]."""
        return _lib.load().pbe_batch_rhs_vjp(self._h, _ptr(N, "N"), _ptr(lam, "lambda"),
                                             _ptr(gN, "gN"), _ptr(gparams, "gparams"),
                                             _ptr(params, "params"), _stream(stream))

    def jvp(self, N, v, out, params, stream=None) -> int:
        """out = J(N) v for every cell (overwritten), J = d RHS / dN."""
        return _lib.load().pbe_batch_jvp(self._h, _ptr(N, "N"), _ptr(v, "v"),
                                         _ptr(params, "params"), _ptr(out, "out"),
                                         _stream(stream))

    def ros2_adaptive(self, N, params, t_end: float, rtol: float = 1e-6, atol: float = 0.0,
                      dt0: float = 1e-3, krylov_dim: int = 16, max_attempts: int = 10000,
                      resid=None, stream=None):
        """ROS2 to t_end with a step size per cell. Returns (code, accepted steps
        per cell, rejected steps per cell, attempts); code 600 (ERR_NOT_READY)
        if max_attempts ran out."""
        steps = np.zeros(self.n_cells, dtype=np.int32)
        rejects = np.zeros(self.n_cells, dtype=np.int32)
        att = ctypes.c_int()
        code = _lib.load().pbe_batch_ros2_adaptive(
            self._h, _ptr(N, "N"), _ptr(params, "params"), float(t_end), float(rtol),
            float(atol), float(dt0), int(krylov_dim), int(max_attempts), steps.ctypes.data,
            rejects.ctypes.data, ctypes.byref(att), _ptr(resid, "resid"), _stream(stream))
        return code, steps, rejects, att.value

    def set_krylov_tol(self, tol: float) -> int:
        """Relative residual that ends a cell's GMRES solve early in ros2 and
        ros2_adaptive (0, the default: krylov_dim steps or an exact breakdown)."""
        return _lib.load().pbe_batch_set_krylov_tol(self._h, float(tol))

    def set_krylov_restarts(self, restarts: int) -> int:
        """Further GMRES cycles (on r - A x) for cells whose residual is above
        the Krylov tolerance after krylov_dim steps (default 0)."""
        return _lib.load().pbe_batch_set_krylov_restarts(self._h, int(restarts))

    def from_soa(self, soa, ld: int, N, stream=None) -> int:
        """N[off_c + i] = soa[i * ld + c] for the bins of every cell (mesh fields
        -> packed state)."""
        return _lib.load().pbe_batch_from_soa(self._h, _ptr(soa, "soa"), int(ld), _ptr(N, "N"),
                                              _stream(stream))

    def to_soa(self, N, soa, ld: int, stream=None) -> int:
        """soa[i * ld + c] = N[off_c + i] for the bins of every cell."""
        return _lib.load().pbe_batch_to_soa(self._h, _ptr(N, "N"), _ptr(soa, "soa"), int(ld),
                                            _stream(stream))

    def ros2(self, N, params, dt: float, n_steps: int, krylov_dim: int = 16, resid=None,
             stream=None) -> int:
        """n_steps linearly implicit ROS2 steps in place on N; each stage's system
        (I - gamma dt J) k = r solved by GMRES(krylov_dim) with Jacobian-vector
        products. resid: optional device array [n_cells], the largest relative
        least-squares residual of the call's solves per cell."""
        return _lib.load().pbe_batch_ros2(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                          float(dt), int(n_steps), int(krylov_dim),
                                          _ptr(resid, "resid") if resid is not None else None,
                                          _stream(stream))

    def tape_forward(self, N, params, dt: float, n_steps: int, checkpoint_every: int,
                     stream=None) -> int:
        """n_steps RK4 steps in place on N with checkpoints for tape_backward."""
        return _lib.load().pbe_batch_tape_forward(self._h, _ptr(N, "N"), _ptr(params, "params"),
                                                  float(dt), int(n_steps), int(checkpoint_every),
                                                  _stream(stream))

    def tape_backward(self, lam_T, gN0, gparams, stream=None) -> int:
        """gN0 = dL/dN(0), gparams[c, j] = dL/d(parameter j of cell c) (overwritten)."""
        return _lib.load().pbe_batch_tape_backward(self._h, _ptr(lam_T, "lambda_T"),
                                                   _ptr(gN0, "gN0"), _ptr(gparams, "gparams"),
                                                   _stream(stream))

    def schedule(self):
        """({class: group size} for the section-count classes present, bundles)."""
        gs = np.zeros(16, dtype=np.int32)
        nb = ctypes.c_int()
        _lib.check(_lib.load().pbe_batch_schedule(self._h, gs.ctypes.data, ctypes.byref(nb)),
                   "pbe_batch_schedule")
        return {c: int(t) for c, t in enumerate(gs) if t}, nb.value

    def split(self, packed: np.ndarray):
        """Per-cell views of a packed host array."""
        return [packed[self.offsets[c]:self.offsets[c + 1]] for c in range(self.n_cells)]

    # -- lifetime ---------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().pbe_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
