// =============================================================================
// pbe_cuda/aggregation.cuh -- C++ drop-in API of libpbe_gb300 (aggregation).
//
// Same namespace, enum values, struct layout/defaults and function signature
// as acuoci/pbe-fixed-pivot-cuda include/pbe_cuda/aggregation.cuh:32-39,
// :59-73, :115-120, so code written against the reference (its tests,
// examples, host ODE/CFD drivers) recompiles unchanged and links against
// libpbe_gb300.so instead. The implementation is the GB300 library; the C ABI
// of the same functions is declared in pbe_gb300.h.
//
//   rhs[i] += sum_{j<=k} (1 - delta_jk/2) beta_jk N_j N_k eta_i(x_j + x_k)
//             - N_i sum_k beta_ik N_k
// with fixed-pivot (Kumar-Ramkrishna) weights eta, sums beyond x[n-1] lumped
// into bin n-1.
// =============================================================================
#pragma once

#include <cuda_runtime.h>

namespace pbe_cuda {

// beta(xj, xk); aj = xj^(1/3).
enum class AggregationKernel : int {
    Constant      = 0,   // beta0
    Sum           = 1,   // beta0 (xj + xk)
    Product       = 2,   // beta0 xj xk
    Brownian      = 3,   // beta_br (aj/ak + ak/aj + 2)
    Shear         = 4,   // beta_sh (aj + ak)^3
    BrownianShear = 5    // Brownian + Shear
};

struct AggregationParams {
    int    n          = 0;     // number of pivots
    double log_x0     = 0.0;   // log(x[0]); accepted, not needed by this library
    double inv_log_r  = 0.0;   // 1/log(r) on a geometric grid, 0 for a generic grid
    AggregationKernel kernel_type = AggregationKernel::Constant;
    double beta0      = 1.0;
    double beta_br    = 0.0;
    double beta_sh    = 0.0;
    int    block_size = 256;   // accepted; <= 0 means 256, > 1024 is rejected
};

// N, x, rhs: device pointers of length n (x strictly positive, increasing).
// rhs must be pre-zeroed; the call adds into it. Asynchronous on `stream`.
// Returns cudaErrorInvalidValue for n <= 0 or a bad enum,
// cudaErrorInvalidDevicePointer for a null pointer, else cudaGetLastError().
cudaError_t launch_aggregation_rhs(
    const double*            N,
    const double*            x,
    double*                  rhs,
    const AggregationParams& params,
    cudaStream_t             stream = 0);

// Adjoint (no counterpart in the reference): with lambda = dL/drhs, adds
// dL/dN into gN[n] and dL/d(beta0, beta_br, beta_sh) into gparams[3] (device).
cudaError_t launch_aggregation_rhs_vjp(
    const double*            N,
    const double*            x,
    const double*            lambda,
    double*                  gN,
    double*                  gparams,
    const AggregationParams& params,
    cudaStream_t             stream = 0);

} // namespace pbe_cuda
