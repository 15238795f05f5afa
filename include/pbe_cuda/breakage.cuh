// =============================================================================
// pbe_cuda/breakage.cuh -- C++ drop-in API of libpbe_gb300 (breakage).
//
// Same namespace, enum values, struct layout/defaults and signature as
// acuoci/pbe-fixed-pivot-cuda include/pbe_cuda/breakage.cuh:30-35, :63-77,
// :122-129.
//
//   rhs[i] += -S(x_i) N_i + sum_j sum_q S(x_j) N_j bw_q eta_i(x_j t_q)
// (terms with S == 0 or N_j <= 2.2e-308 are skipped; fragments at or below
// x[0] go to bin 0, at or above x[n-1] to bin n-1).
//
// Daughter distributions are encoded by the caller as (t_q, bw_q) tables:
//   symmetric binary : n_quad = 1, t_q = {0.5},        bw_q = {2}
//   erosion (eps)    : n_quad = 2, t_q = {1-eps, eps}, bw_q = {1, 1}
//   uniform          : Gauss-Legendre on (0,1),        bw_q = 2 w_q
//   power law (p)    : two-interval Gauss-Legendre,    bw_q = (p+2) t_q^p w_q
// The Python package pbe_gb300.quadrature builds all four.
// =============================================================================
#pragma once

#include <cuda_runtime.h>

namespace pbe_cuda {

enum class BreakageSelection : int {
    Constant  = 0,   // S0
    Linear    = 1,   // S0 v / v_ref
    PowerLaw  = 2,   // S0 (v / v_ref)^alpha
    Threshold = 3    // v > v_min ? S0 : 0
};

struct BreakageParams {
    int    n      = 0;
    int    n_quad = 0;
    BreakageSelection selection = BreakageSelection::Constant;
    double S0     = 1.0;
    double v_ref  = 1.0;
    double alpha  = 1.0;
    double v_min  = 0.0;
    int    block_size = 256;   // accepted; must be 1..1024
};

// N, x, rhs: device arrays of length n; t_q, bw_q: device arrays of length
// n_quad. rhs must be pre-zeroed; the call adds into it.
// Returns cudaErrorInvalidValue for n <= 0, n_quad <= 0, a bad enum or
// block_size <= 0, cudaErrorInvalidDevicePointer for a null pointer, else
// cudaGetLastError().
cudaError_t launch_breakage_rhs(
    const double*          N,
    const double*          x,
    const double*          t_q,
    const double*          bw_q,
    double*                rhs,
    const BreakageParams&  params,
    cudaStream_t           stream = 0);

// Adjoint (no counterpart in the reference): with lambda = dL/drhs, adds
// dL/dN into gN[n] and dL/d(S0, v_ref, alpha, v_min) into gparams[4] (device).
cudaError_t launch_breakage_rhs_vjp(
    const double*          N,
    const double*          x,
    const double*          t_q,
    const double*          bw_q,
    const double*          lambda,
    double*                gN,
    double*                gparams,
    const BreakageParams&  params,
    cudaStream_t           stream = 0);

} // namespace pbe_cuda
