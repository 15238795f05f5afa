"""Checkpointed RK4 adjoint of one instance (C ABI pbe_rk4_tape_*).

    tape = Rk4Tape(n_steps, dt, every, agg_sets=[AggregationParams...],
                   brk_sets=[BreakageParams...], step_set=[...])
    tape.forward(N, x, t_q, bw_q)          # N(0) -> N(T) in place, checkpoints kept
    tape.backward(lam_T, gN0, g_agg, g_brk)  # dL/dN(0), dL/d(parameters per set)

Arrays are float64 CUDA tensors or device addresses; the calls are
asynchronous on `stream` and return the cudaError_t code.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import AggregationParams, BreakageParams, PbeError
from .rhs import _ptr, _stream


class Rk4Tape:
    def __init__(self, n_steps: int, dt: float, checkpoint_every: int,
                 agg_sets: Optional[Sequence[AggregationParams]] = None,
                 brk_sets: Optional[Sequence[BreakageParams]] = None,
                 step_set: Optional[Sequence[int]] = None):
        lib = _lib.load()
        n_sets = len(agg_sets if agg_sets is not None else brk_sets or [])
        self._agg = None if agg_sets is None else (AggregationParams * n_sets)(*agg_sets)
        self._brk = None if brk_sets is None else (BreakageParams * n_sets)(*brk_sets)
        ss = None if step_set is None else np.ascontiguousarray(step_set, dtype=np.int32)
        h = ctypes.c_void_p()
        code = lib.pbe_rk4_tape_create(
            ctypes.byref(h), int(n_steps), float(dt), int(checkpoint_every), n_sets,
            None if self._agg is None else ctypes.addressof(self._agg),
            None if self._brk is None else ctypes.addressof(self._brk),
            None if ss is None else ss.ctypes.data)
        if code:
            raise PbeError(code, "pbe_rk4_tape_create")
        self._h = h
        self.n_sets = n_sets

    def forward(self, N, x, t_q=None, bw_q=None, stream=None) -> int:
        return _lib.load().pbe_rk4_tape_forward(self._h, _ptr(N, "N"), _ptr(x, "x"),
                                                _ptr(t_q, "t_q"), _ptr(bw_q, "bw_q"),
                                                _stream(stream))

    def backward(self, lam_T, gN0, g_agg=None, g_brk=None, stream=None) -> int:
        return _lib.load().pbe_rk4_tape_backward(self._h, _ptr(lam_T, "lambda_T"),
                                                 _ptr(gN0, "gN0"), _ptr(g_agg, "g_agg"),
                                                 _ptr(g_brk, "g_brk"), _stream(stream))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().pbe_rk4_tape_destroy(self._h)
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
