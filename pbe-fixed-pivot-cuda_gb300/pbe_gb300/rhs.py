"""Python mirror of the pbe_cuda operator interface.

`aggregation_rhs` and `breakage_rhs` have the argument meaning, accumulation
rule (rhs is added to, never overwritten) and return codes of the reference's
`pbe_cuda::launch_aggregation_rhs` / `launch_breakage_rhs`
(acuoci/pbe-fixed-pivot-cuda include/pbe_cuda/aggregation.cuh:115-120,
include/pbe_cuda/breakage.cuh:122-129): they return the cudaError_t value as
an int and do not synchronise. Arrays are torch CUDA tensors (float64,
contiguous) or raw device addresses (int); torch only supplies device memory
and the stream.
"""
from __future__ import annotations

from typing import Optional, Union

from . import _lib
from ._lib import AggregationParams, BreakageParams, MODE_DEFAULT

Array = Union["torch.Tensor", int, None]  # noqa: F821


def _ptr(a: Array, name: str) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, int):
        return a or None
    import torch

    if not isinstance(a, torch.Tensor):
        raise TypeError("%s must be a torch tensor or a device address" % name)
    if a.dtype != torch.float64:
        raise TypeError("%s must be float64 (got %s)" % (name, a.dtype))
    if not a.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if not a.is_contiguous():
        raise TypeError("%s must be contiguous" % name)
    return a.data_ptr()


def _stream(stream) -> Optional[int]:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream or None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def aggregation_rhs(N: Array, x: Array, rhs: Array, params: AggregationParams, stream=None,
                    mode: int = MODE_DEFAULT, workspace: Array = None,
                    workspace_bytes: int = 0) -> int:
    """rhs += aggregation term. Returns the cudaError_t code (0 = success)."""
    lib = _lib.load()
    ws = None
    if workspace is not None:
        import torch

        if isinstance(workspace, torch.Tensor):
            workspace_bytes = workspace.numel() * workspace.element_size()
            ws = workspace.data_ptr()
        else:
            ws = int(workspace)
    if mode == MODE_DEFAULT and ws is None:
        return lib.pbe_aggregation_rhs(_ptr(N, "N"), _ptr(x, "x"), _ptr(rhs, "rhs"),
                                       params, _stream(stream))
    return lib.pbe_aggregation_rhs_ex(_ptr(N, "N"), _ptr(x, "x"), _ptr(rhs, "rhs"), params,
                                      int(mode), ws, int(workspace_bytes), _stream(stream))


def breakage_rhs(N: Array, x: Array, t_q: Array, bw_q: Array, rhs: Array,
                 params: BreakageParams, stream=None, mode: int = MODE_DEFAULT,
                 workspace: Array = None, workspace_bytes: int = 0) -> int:
    """rhs += breakage term. Returns the cudaError_t code (0 = success)."""
    lib = _lib.load()
    ws = None
    if workspace is not None:
        import torch

        if isinstance(workspace, torch.Tensor):
            workspace_bytes = workspace.numel() * workspace.element_size()
            ws = workspace.data_ptr()
        else:
            ws = int(workspace)
    if mode == MODE_DEFAULT and ws is None:
        return lib.pbe_breakage_rhs(_ptr(N, "N"), _ptr(x, "x"), _ptr(t_q, "t_q"),
                                    _ptr(bw_q, "bw_q"), _ptr(rhs, "rhs"), params, _stream(stream))
    return lib.pbe_breakage_rhs_ex(_ptr(N, "N"), _ptr(x, "x"), _ptr(t_q, "t_q"),
                                   _ptr(bw_q, "bw_q"), _ptr(rhs, "rhs"), params, int(mode), ws,
                                   int(workspace_bytes), _stream(stream))


def aggregation_workspace_bytes(n: int, mode: int = MODE_DEFAULT) -> int:
    return int(_lib.load().pbe_aggregation_workspace_bytes(int(n), int(mode)))


def breakage_workspace_bytes(n: int, n_quad: int, mode: int = MODE_DEFAULT) -> int:
    return int(_lib.load().pbe_breakage_workspace_bytes(int(n), int(n_quad), int(mode)))


def aggregation_rhs_vjp(N: Array, x: Array, lam: Array, gN: Array, gparams: Array,
                        params: AggregationParams, stream=None) -> int:
    """gN += dL/dN, gparams[0:3] += dL/d(beta0, beta_br, beta_sh) for L = lam . rhs_agg."""
    return _lib.load().pbe_aggregation_rhs_vjp(_ptr(N, "N"), _ptr(x, "x"), _ptr(lam, "lambda"),
                                               _ptr(gN, "gN"), _ptr(gparams, "gparams"), params,
                                               None, 0, _stream(stream))


def breakage_rhs_vjp(N: Array, x: Array, t_q: Array, bw_q: Array, lam: Array, gN: Array,
                     gparams: Array, params: BreakageParams, stream=None) -> int:
    """gN += dL/dN, gparams[0:4] += dL/d(S0, v_ref, alpha, v_min) for L = lam . rhs_brk."""
    return _lib.load().pbe_breakage_rhs_vjp(_ptr(N, "N"), _ptr(x, "x"), _ptr(t_q, "t_q"),
                                            _ptr(bw_q, "bw_q"), _ptr(lam, "lambda"), _ptr(gN, "gN"),
                                            _ptr(gparams, "gparams"), params, None, 0,
                                            _stream(stream))
