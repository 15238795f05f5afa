/*
 * pbe_gb300.h -- C ABI of the GB300 (sm_103a) fixed-pivot population-balance
 * right-hand side library (libpbe_gb300.so).
 *
 * Plain pointers, sizes and POD structs only: no CUDA or C++ types appear in
 * the signatures, so any FFI (ctypes, cgo, JNI, N-API, Fortran ISO_C_BINDING)
 * can bind it. Streams are passed as void* and are cudaStream_t handles
 * (NULL = legacy default stream). Every function returns a cudaError_t value
 * as int: 0 success, 1 cudaErrorInvalidValue, 17 cudaErrorInvalidDevicePointer,
 * 9 cudaErrorInvalidConfiguration, 2 cudaErrorMemoryAllocation, or whatever
 * cudaGetLastError() reports after the launches (which, like the reference,
 * also surfaces and clears an earlier sticky error). Nothing synchronises;
 * device faults show up at the caller's next synchronisation.
 *
 * All N / x / rhs / t_q / bw_q pointers are DEVICE pointers owned by the
 * caller. rhs must be zeroed (or hold other source terms) before the call:
 * the functions ADD their contribution, so aggregation and breakage can share
 * one rhs. Concurrent calls on different streams with disjoint rhs are safe.
 *
 * Reference interfaces replaced (acuoci/pbe-fixed-pivot-cuda):
 *   pbe_agg_params_t       <- pbe_cuda::AggregationParams  include/pbe_cuda/aggregation.cuh:59-73
 *   pbe_brk_params_t       <- pbe_cuda::BreakageParams     include/pbe_cuda/breakage.cuh:63-77
 *   pbe_aggregation_rhs    <- pbe_cuda::launch_aggregation_rhs  include/pbe_cuda/aggregation.cuh:115-120
 *   pbe_breakage_rhs       <- pbe_cuda::launch_breakage_rhs     include/pbe_cuda/breakage.cuh:122-129
 * The structs have the same member order, types and therefore the same layout
 * as the reference's C++ structs (enum class : int members become int).
 */
#ifndef PBE_GB300_H
#define PBE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Aggregation frequency (values of pbe_cuda::AggregationKernel, aggregation.cuh:32-39). */
enum {
    PBE_AGG_CONSTANT       = 0,  /* beta0                                   */
    PBE_AGG_SUM            = 1,  /* beta0 (xj + xk)                         */
    PBE_AGG_PRODUCT        = 2,  /* beta0 xj xk                             */
    PBE_AGG_BROWNIAN       = 3,  /* beta_br (aj/ak + ak/aj + 2), a = x^(1/3) */
    PBE_AGG_SHEAR          = 4,  /* beta_sh (aj + ak)^3                     */
    PBE_AGG_BROWNIAN_SHEAR = 5   /* Brownian + Shear                        */
};

/* Selection function (values of pbe_cuda::BreakageSelection, breakage.cuh:30-35). */
enum {
    PBE_SEL_CONSTANT  = 0,  /* S0                        */
    PBE_SEL_LINEAR    = 1,  /* S0 v / v_ref              */
    PBE_SEL_POWERLAW  = 2,  /* S0 (v / v_ref)^alpha      */
    PBE_SEL_THRESHOLD = 3   /* v > v_min ? S0 : 0        */
};

/* Birth accumulation mode.
 *   GATHER  : every output bin is reduced by one owner in a fixed order, no
 *             atomics; results are bitwise identical run to run.
 *   SCATTER : work tiles flush partial sums with FP64 atomicAdd; the order of
 *             the flushes (and hence the last bits) can vary run to run.
 *   DEFAULT : GATHER unless the environment variable PBE_GB300_MODE is
 *             "scatter" (read once per process). */
enum { PBE_MODE_DEFAULT = 0, PBE_MODE_SCATTER = 1, PBE_MODE_GATHER = 2 };

typedef struct pbe_agg_params {
    int    n;            /* number of pivots (length of N, x, rhs)             */
    double log_x0;       /* log(x[0]) (accepted for API compatibility)         */
    double inv_log_r;    /* 1/log(x1/x0) for a geometric grid, 0 for generic   */
    int    kernel_type;  /* PBE_AGG_*                                          */
    double beta0;        /* Constant / Sum / Product prefactor                 */
    double beta_br;      /* Brownian prefactor                                 */
    double beta_sh;      /* shear prefactor                                    */
    int    block_size;   /* accepted for compatibility; <= 0 means 256, > 1024 is rejected */
} pbe_agg_params_t;

typedef struct pbe_brk_params {
    int    n;            /* number of pivots                                   */
    int    n_quad;       /* quadrature points per parent (length of t_q, bw_q) */
    int    selection;    /* PBE_SEL_*                                          */
    double S0;           /* selection prefactor                                */
    double v_ref;        /* reference volume (Linear, PowerLaw)                */
    double alpha;        /* power-law exponent (PowerLaw)                      */
    double v_min;        /* threshold volume (Threshold: S = 0 for v <= v_min) */
    int    block_size;   /* accepted for compatibility; must be 1..1024        */
} pbe_brk_params_t;

/* ---------------------------------------------------------------------------
 * Drop-in entry points (reference call semantics, default mode).
 * They take their scratch space from a library-private, stream-ordered CUDA
 * memory pool (cudaMallocFromPoolAsync / cudaFreeAsync on `stream`).
 * ------------------------------------------------------------------------- */

/* rhs += aggregation source term. Replaces pbe_cuda::launch_aggregation_rhs
 * (reference include/pbe_cuda/aggregation.cuh:115-120, src/aggregation.cu:16-61). */
int pbe_aggregation_rhs(const double* N, const double* x, double* rhs,
                        const pbe_agg_params_t* params, void* stream);

/* rhs += breakage source term (death then quadrature birth). Replaces
 * pbe_cuda::launch_breakage_rhs (reference include/pbe_cuda/breakage.cuh:122-129,
 * src/breakage.cu:14-79). */
int pbe_breakage_rhs(const double* N, const double* x, const double* t_q,
                     const double* bw_q, double* rhs,
                     const pbe_brk_params_t* params, void* stream);

/* ---------------------------------------------------------------------------
 * Explicit-mode / explicit-workspace variants (no reference counterpart; the
 * reference has one mode and no scratch). With workspace == NULL they
 * allocate from the pool like the drop-in calls; otherwise `workspace` must be
 * a device buffer of at least the queried size, 256-byte aligned, used by no
 * other call in flight. The *_workspace_bytes queries are host-only.
 * ------------------------------------------------------------------------- */
size_t pbe_aggregation_workspace_bytes(int n, int mode);
size_t pbe_breakage_workspace_bytes(int n, int n_quad, int mode);

int pbe_aggregation_rhs_ex(const double* N, const double* x, double* rhs,
                           const pbe_agg_params_t* params, int mode,
                           void* workspace, size_t workspace_bytes,
                           void* stream);

int pbe_breakage_rhs_ex(const double* N, const double* x, const double* t_q,
                        const double* bw_q, double* rhs,
                        const pbe_brk_params_t* params, int mode,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Aggregation without any allocation (no counterpart in the reference, whose
 * kernels need no scratch). For host codes that cannot let a library allocate
 * device memory -- solvers that give the whole GPU to their own allocator,
 * codes that forbid allocation once time stepping starts, plug-in interfaces
 * with no way to pass a workspace -- this runs the same kernels as
 * pbe_aggregation_rhs_ex with its scratch in a fixed device array compiled
 * into the library (about 1.9 MiB, held by every GPU that loads the library).
 *   Limit: params->n <= 32768; larger n returns cudaErrorInvalidValue.
 *   The first call on a device looks up that array's address; make it before
 *   any stream capture starts.
 *   All calls on a device share the array: calls whose kernels overlap on the
 *   GPU race; order them on one stream. Nothing needs clearing between calls.
 * mode: PBE_MODE_*. Same argument checks and return codes as
 * pbe_aggregation_rhs. */
int pbe_aggregation_rhs_noalloc(const double* N, const double* x, double* rhs,
                                const pbe_agg_params_t* params, int mode, void* stream);

/* ---------------------------------------------------------------------------
 * Vector-Jacobian products (no counterpart in the reference). Given
 * lambda = dL/drhs (device, length n) they ADD dL/dN into gN (length n) and
 * dL/d(parameters) into gparams (device):
 *   aggregation: gparams[0..2] += dL/dbeta0, dL/dbeta_br, dL/dbeta_sh
 *   breakage:    gparams[0..3] += dL/dS0, dL/dv_ref, dL/dalpha, dL/dv_min (= 0)
 * The result is bitwise reproducible. workspace: NULL (pool) or a device
 * buffer of pbe_vjp_workspace_bytes(n), 256-byte aligned. Same argument
 * checks as the forward calls (lambda and gparams must be non-null).
 * ------------------------------------------------------------------------- */
size_t pbe_vjp_workspace_bytes(int n);

int pbe_aggregation_rhs_vjp(const double* N, const double* x, const double* lambda,
                            double* gN, double* gparams, const pbe_agg_params_t* params,
                            void* workspace, size_t workspace_bytes, void* stream);

int pbe_breakage_rhs_vjp(const double* N, const double* x, const double* t_q,
                         const double* bw_q, const double* lambda, double* gN,
                         double* gparams, const pbe_brk_params_t* params,
                         void* workspace, size_t workspace_bytes, void* stream);

/* Human-readable name of a return code (cudaGetErrorString). */
const char* pbe_error_string(int code);

/* Library version, e.g. 100 for 0.1.0. */
int pbe_version(void);

/* Profiling aid (no reference counterpart): when start and stop are both
 * non-NULL cudaEvent_t handles, every aggregation call records `start` just
 * before and `stop` just after its pair kernel, on the call's stream, so a
 * caller can time that kernel alone with cudaEventElapsedTime. NULL, NULL
 * turns it off. Process-wide setting; not for concurrent use. Returns 0. */
int pbe_set_profile_events(void* start, void* stop);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PBE_GB300_H */
