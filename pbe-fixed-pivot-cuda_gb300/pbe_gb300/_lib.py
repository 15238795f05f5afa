"""ctypes binding of libpbe_gb300.so (the C ABI declared in include/pbe_gb300.h).

The Python layer only marshals arguments: every RHS evaluation runs in the
library's sm_103a kernels. If the shared library is missing the import fails
with an error telling how to build it -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

_PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# PBE_GB300_LIB selects another build of the library (e.g. one compiled with
# different tuning macros); default: the in-tree build.
LIB_PATH = os.environ.get("PBE_GB300_LIB") or os.path.join(_PKG_DIR, "lib", "libpbe_gb300.so")

# cudaError_t values used by the API
SUCCESS = 0
ERR_INVALID_VALUE = 1
ERR_MEMORY_ALLOCATION = 2
ERR_INVALID_CONFIGURATION = 9
ERR_INVALID_DEVICE_POINTER = 17
ERR_NOT_READY = 600

# enum values (include/pbe_gb300.h, identical to the reference's enums)
AGG_CONSTANT, AGG_SUM, AGG_PRODUCT, AGG_BROWNIAN, AGG_SHEAR, AGG_BROWNIAN_SHEAR = range(6)
SEL_CONSTANT, SEL_LINEAR, SEL_POWERLAW, SEL_THRESHOLD = range(4)
MODE_DEFAULT, MODE_SCATTER, MODE_GATHER = 0, 1, 2


class AggregationParams(ctypes.Structure):
    """Layout of pbe_agg_params_t == pbe_cuda::AggregationParams
    (reference include/pbe_cuda/aggregation.cuh:59-73), same defaults."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("log_x0", ctypes.c_double),
        ("inv_log_r", ctypes.c_double),
        ("kernel_type", ctypes.c_int),
        ("beta0", ctypes.c_double),
        ("beta_br", ctypes.c_double),
        ("beta_sh", ctypes.c_double),
        ("block_size", ctypes.c_int),
    ]

    def __init__(self, **kw):
        defaults = dict(n=0, log_x0=0.0, inv_log_r=0.0, kernel_type=AGG_CONSTANT, beta0=1.0,
                        beta_br=0.0, beta_sh=0.0, block_size=256)
        defaults.update(kw)
        super().__init__(**defaults)


class BreakageParams(ctypes.Structure):
    """Layout of pbe_brk_params_t == pbe_cuda::BreakageParams
    (reference include/pbe_cuda/breakage.cuh:63-77), same defaults."""

    _fields_ = [
        ("n", ctypes.c_int),
        ("n_quad", ctypes.c_int),
        ("selection", ctypes.c_int),
        ("S0", ctypes.c_double),
        ("v_ref", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("v_min", ctypes.c_double),
        ("block_size", ctypes.c_int),
    ]

    def __init__(self, **kw):
        defaults = dict(n=0, n_quad=0, selection=SEL_CONSTANT, S0=1.0, v_ref=1.0, alpha=1.0,
                        v_min=0.0, block_size=256)
        defaults.update(kw)
        super().__init__(**defaults)


class BatchCellParams(ctypes.Structure):
    """Layout of pbe_batch_cell_params_t (one per cell of a batch plan)."""

    _fields_ = [(name, ctypes.c_double) for name in
                ("beta0", "beta_br", "beta_sh", "S0", "v_ref", "alpha", "v_min", "reserved")]


BATCH_TUNE, BATCH_RETUNE = 1, 2
BATCH_BRK_PREP, BATCH_BRK_TASKS = 4, 8
DEATH_MOMENTS, DEATH_DMMA = 0, 1
DAUGHTER_SYMMETRIC, DAUGHTER_EROSION, DAUGHTER_UNIFORM, DAUGHTER_POWERLAW = range(4)

_P = ctypes.c_void_p
_I = ctypes.c_int
_SIGNATURES = {
    "pbe_aggregation_rhs": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(AggregationParams), _P]),
    "pbe_breakage_rhs": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(BreakageParams), _P]),
    "pbe_aggregation_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "pbe_breakage_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "pbe_aggregation_rhs_ex": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(AggregationParams),
                                              ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "pbe_breakage_rhs_ex": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(BreakageParams),
                                           ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "pbe_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pbe_version": (ctypes.c_int, []),
    "pbe_set_profile_events": (ctypes.c_int, [_P, _P]),
    "pbe_scratch_pool_usage": (ctypes.c_int, [ctypes.POINTER(ctypes.c_ulonglong),
                                              ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
    "pbe_vjp_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int]),
    "pbe_aggregation_rhs_vjp": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(AggregationParams),
                                               _P, ctypes.c_size_t, _P]),
    "pbe_breakage_rhs_vjp": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(BreakageParams),
                                            _P, ctypes.c_size_t, _P]),
    "pbe_batch_create": (_I, [ctypes.POINTER(_P), _I, _P, _P, _I, _P, _P, _I, _I, _I, _P, _P, _I, _P]),
    "pbe_batch_destroy": (_I, [_P]),
    "pbe_batch_offsets": (_I, [_P, _P]),
    "pbe_batch_rhs": (_I, [_P, _P, _P, _P, _P]),
    "pbe_batch_rk4": (_I, [_P, _P, _P, ctypes.c_double, _I, _P]),
    "pbe_batch_rk4_percell": (_I, [_P, _P, _P, ctypes.c_double, _I, _P]),
    "pbe_batch_rk4_prepare": (_I, [_P, _P, _P, ctypes.c_double, _I]),
    "pbe_batch_schedule": (_I, [_P, _P, _P]),
    "pbe_batch_death": (_I, [_P, _P, _P, _P, _I, _P]),
    "pbe_batch_rhs_vjp": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "pbe_batch_rk45": (_I, [_P, _P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_double, _I, _P, _P, _P, _P]),
    "pbe_batch_jvp": (_I, [_P, _P, _P, _P, _P, _P]),
    "pbe_batch_from_soa": (_I, [_P, _P, ctypes.c_longlong, _P, _P]),
    "pbe_batch_ros2_adaptive": (_I, [_P, _P, _P, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, _I, _I, _P, _P, _P, _P,
                                     _P]),
    "pbe_batch_to_soa": (_I, [_P, _P, _P, ctypes.c_longlong, _P]),
    "pbe_batch_ros2": (_I, [_P, _P, _P, ctypes.c_double, _I, _I, _P, _P]),
    "pbe_batch_set_krylov_tol": (_I, [_P, ctypes.c_double]),
    "pbe_batch_set_krylov_restarts": (_I, [_P, _I]),
    "pbe_daughter_table": (_I, [_I, _I, ctypes.c_double, ctypes.c_double, _P, _P, _I, _P]),
    "pbe_batch_tape_forward": (_I, [_P, _P, _P, ctypes.c_double, _I, _I, _P]),
    "pbe_batch_tape_backward": (_I, [_P, _P, _P, _P, _P]),
    "pbe_rk4_tape_create": (_I, [ctypes.POINTER(_P), _I, ctypes.c_double, _I, _I, _P, _P, _P]),
    "pbe_rk4_tape_destroy": (_I, [_P]),
    "pbe_rk4_tape_forward": (_I, [_P, _P, _P, _P, _P, _P]),
    "pbe_rk4_tape_backward": (_I, [_P, _P, _P, _P, _P, _P]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load (once) and return the shared library, with argument types set."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise ImportError(
            "libpbe_gb300.so not found at %s; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python pbe-fixed-pivot-cuda_gb300/build.py`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def scratch_pool_usage(reset_high: bool = False) -> tuple[int, int]:
    """(bytes the library's scratch pool reserves on the current device,
    high-water mark of its bytes in use); reset_high clears the mark after
    reading it."""
    r, h = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
    check(load().pbe_scratch_pool_usage(ctypes.byref(r), ctypes.byref(h), int(reset_high)),
          "scratch pool usage")
    return int(r.value), int(h.value)


def error_string(code: int) -> str:
    return load().pbe_error_string(int(code)).decode()


class PbeError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = int(code)
        super().__init__("%s%s (cudaError %d)" % (what + ": " if what else "", error_string(code), code))


def check(code: int, what: str = "") -> None:
    """Raise PbeError unless code == 0."""
    if code != SUCCESS:
        raise PbeError(code, what)
