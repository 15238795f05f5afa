"""pbe_gb300 -- GB300 (sm_103a) fixed-pivot population-balance RHS.

Python face of libpbe_gb300.so. The operator interface mirrors the reference
pbe_cuda API (AggregationParams / BreakageParams, aggregation_rhs /
breakage_rhs adding into a pre-zeroed rhs and returning a cudaError_t code).
"""
from ._lib import (  # noqa: F401
    AGG_BROWNIAN,
    AGG_BROWNIAN_SHEAR,
    AGG_CONSTANT,
    AGG_PRODUCT,
    AGG_SHEAR,
    AGG_SUM,
    ERR_INVALID_CONFIGURATION,
    ERR_INVALID_DEVICE_POINTER,
    ERR_NOT_READY,
    ERR_INVALID_VALUE,
    LIB_PATH,
    MODE_DEFAULT,
    MODE_GATHER,
    MODE_SCATTER,
    SEL_CONSTANT,
    SEL_LINEAR,
    SEL_POWERLAW,
    SEL_THRESHOLD,
    BATCH_BRK_PREP,
    BATCH_BRK_TASKS,
    BATCH_RETUNE,
    BATCH_TUNE,
    DEATH_DMMA,
    DEATH_MOMENTS,
    AggregationParams,
    BatchCellParams,
    BreakageParams,
    PbeError,
    check,
    error_string,
    scratch_pool_usage,
    load,
)
from .rhs import (  # noqa: F401
    aggregation_rhs,
    aggregation_rhs_vjp,
    aggregation_workspace_bytes,
    breakage_rhs,
    breakage_rhs_vjp,
    breakage_workspace_bytes,
)
from .adjoint import Rk4Tape  # noqa: F401
from .batch import BatchPlan  # noqa: F401
from . import grids, quadrature  # noqa: F401

__version__ = "0.1.0"
