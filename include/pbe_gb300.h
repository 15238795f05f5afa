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
 * into the library (about 8.5 MiB, held by every GPU that loads the library).
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

/* ---------------------------------------------------------------------------
 * Batched cells (no counterpart in the reference, whose callers loop over
 * cells and launch per cell and per RK4 stage, with host round trips between
 * stages: examples/common/pbe_examples_utils.hpp:409-456, driven per time
 * step as in examples/flocculation_two_stage/main.cpp:311-355).
 *
 * A plan describes n_cells independent PBE instances ("cells"). Cell c has
 * cell_n[c] sections on the first cell_n[c] pivots of grid cell_grid[c]. The
 * n_grids grids are given packed, grid after grid, in grid_x (grid g has
 * grid_n[g] strictly increasing positive pivots). Cells that share a grid
 * share its tables, which are built once per plan. All cells use one
 * aggregation kernel type (PBE_AGG_*, or -1 for none) and one breakage
 * selection (PBE_SEL_*, or -1 for none) with one daughter table (n_quad
 * points, 0 < t_q <= 1); each cell has its own coefficients, read from a
 * device array of pbe_batch_cell_params_t at every call.
 *
 * Packed cell state: cell c owns entries [off_c, off_c + cell_n[c]) of N and
 * rhs, off = exclusive prefix sum of cell_n in cell order (pbe_batch_offsets).
 *
 * Results are those of the single-instance functions on each cell (same
 * formulas, same clip rules) up to the order of FP64 summation; for one plan
 * they are bitwise reproducible run to run (no atomics on the data path).
 *
 * The plan owns device memory for its tables, its task schedule and its stage
 * arrays (about 7 doubles per packed bin) and caches one CUDA graph. Use a
 * plan from one stream at a time. The plan-creation arrays are HOST arrays;
 * the call arrays (N, rhs, params) are DEVICE arrays.
 * ------------------------------------------------------------------------- */
typedef struct pbe_batch_plan* pbe_batch_t;

typedef struct pbe_batch_cell_params {
    double beta0, beta_br, beta_sh;    /* aggregation coefficients (pbe_agg_params_t)   */
    double S0, v_ref, alpha, v_min;    /* selection parameters (pbe_brk_params_t)       */
    double reserved;                   /* set to 0                                      */
} pbe_batch_cell_params_t;

/* flags of pbe_batch_create */
enum {
    PBE_BATCH_TUNE   = 1,  /* pick the tile group size per section-count class by timing
                              candidates on the device (results cached per process, and
                              in the file named by PBE_GB300_TUNE_CACHE when set)        */
    PBE_BATCH_RETUNE = 2,  /* like TUNE, ignoring cached results                          */
    /* where the breakage term is gathered (bitwise the same result either way);
     * default: by the pair tasks for plans of at most 2 x SM-count cells, by a
     * per-cell prep CTA otherwise */
    PBE_BATCH_BRK_PREP  = 4,   /* always by the per-cell prep CTA                        */
    PBE_BATCH_BRK_TASKS = 8    /* always by the pair tasks, each for its own bins         */
};

/* Builds a plan. Returns 1 (InvalidValue) for inconsistent sizes, a cell with
 * more sections than its grid, non-increasing or non-positive pivots, or t_q
 * outside (0, 1]; 2 (MemoryAllocation) when device memory runs out. */
int pbe_batch_create(pbe_batch_t* plan, int n_grids, const int* grid_n, const double* grid_x,
                     int n_cells, const int* cell_n, const int* cell_grid, int kernel_type,
                     int selection, int n_quad, const double* t_q, const double* bw_q,
                     int flags, void* stream);

/* Frees the plan and its device memory (cudaFree waits for device work in
 * flight). NULL is accepted. */
int pbe_batch_destroy(pbe_batch_t plan);

/* offsets (host, n_cells + 1 entries) receives the packed offsets; the last
 * entry is the packed length. */
int pbe_batch_offsets(pbe_batch_t plan, long long* offsets);

/* rhs += RHS(N) for every cell (aggregation + breakage). */
int pbe_batch_rhs(pbe_batch_t plan, const double* N, double* rhs,
                  const pbe_batch_cell_params_t* params, void* stream);

/* n_steps classical RK4 steps of size dt on every cell, in place on N, as one
 * CUDA graph launch (captured on the first call and reused while N, params,
 * dt and n_steps stay the same). The stage arithmetic is that of the
 * reference examples' rk4_step (pbe_examples_utils.hpp:416-456). */
int pbe_batch_rk4(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                  double dt, int n_steps, void* stream);

/* Captures and instantiates the graph pbe_batch_rk4 would launch for these
 * arguments, without running it (so that a timed or latency-critical first
 * call does not pay for the capture). */
int pbe_batch_rk4_prepare(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                          double dt, int n_steps);

/* The same integration as a per-cell launch loop: for every step, cell and
 * stage, the single-instance aggregation and breakage calls plus a stage
 * update kernel (no graph, no batching). Baseline and cross-check. */
int pbe_batch_rk4_percell(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                          double dt, int n_steps, void* stream);

/* Aggregation death term of every cell, death[off_c + i] =
 * N_ci sum_k beta_c(x_i, x_k) N_ck (overwritten; the RHS subtracts it), by
 *   PBE_DEATH_MOMENTS: five per-cell moments (the form the RHS kernels use);
 *   PBE_DEATH_DMMA:    a GEMM per grid over the cells sharing it, on the FP64
 *                      tensor cores (mma.sync f64), one per separable term.
 * For comparison and for callers that want the death term alone; needs an
 * aggregation kernel in the plan. */
enum { PBE_DEATH_MOMENTS = 0, PBE_DEATH_DMMA = 1 };
int pbe_batch_death(pbe_batch_t plan, const double* N, const pbe_batch_cell_params_t* params,
                    double* death, int method, void* stream);

/* Adaptive integration of every cell from its current N to t_end (time 0 to
 * t_end) with the embedded Dormand-Prince 5(4) pair, each cell with its own
 * step size: error = RMS over the cell's bins of the embedded estimate over
 * atol + rtol max(|N|, |N_new|); a step is accepted when error <= 1, the next
 * step is dt (0.9 error^(-1/5)) clipped to [0.2, 5] dt (<= dt after a
 * rejection) and to the time left; first step dt0. Everything runs on the
 * device; the host reads one counter every 8 attempts. steps / rejects (host,
 * n_cells, nullable) receive the accepted / rejected steps per cell, *attempts
 * the attempts made. Returns cudaErrorNotReady (600) when some cell has not
 * reached t_end within max_attempts (its N is the state it reached). No
 * counterpart in the reference (its examples step RK4 on the host). */
int pbe_batch_rk45(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                   double t_end, double rtol, double atol, double dt0, int max_attempts,
                   int* steps, int* rejects, int* attempts, void* stream);

/* Vector-Jacobian product of the batched RHS: for L = sum over cells of
 * lambda . rhs(N), gN += dL/dN (packed like N) and
 * gparams[8 c + j] += dL/d(parameter j of cell c), j = beta0, beta_br,
 * beta_sh, S0, v_ref, alpha, v_min (0: threshold step), 7 unused. Same
 * formulas as pbe_aggregation_rhs_vjp / pbe_breakage_rhs_vjp per cell;
 * bitwise reproducible for one plan. */
int pbe_batch_rhs_vjp(pbe_batch_t plan, const double* N, const double* lambda, double* gN,
                      double* gparams, const pbe_batch_cell_params_t* params, void* stream);

/* Checkpointed RK4 adjoint of every cell of a plan (the batched form of
 * pbe_rk4_tape_*). Forward: n_steps RK4 steps in place on N (N(0) -> N(T)),
 * saving N every checkpoint_every steps in plan-owned memory (grown on first
 * use: (n_steps / every + 4 every + 5) packed vectors). Backward, given
 * lambda_T = dL/dN(T) (packed): gN0 = dL/dN(0) and gparams[8 c + j] =
 * dL/d(parameter j of cell c) over the whole run (both overwritten). params
 * (device) must stay unchanged between the two calls. */
int pbe_batch_tape_forward(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                           double dt, int n_steps, int checkpoint_every, void* stream);
int pbe_batch_tape_backward(pbe_batch_t plan, const double* lambda_T, double* gN0,
                            double* gparams, void* stream);

/* Jacobian-vector product of the batched RHS: out = J(N) v for every cell
 * (packed like N; overwritten), J = d rhs / dN of aggregation plus breakage.
 * Aggregation is quadratic in N, so J(N) v = T(N, v) + T(v, N) with T(a, b)
 * the pair sum of src/aggregation_kernels.cuh:145-239 with the rate
 * beta a_j b_k (1/2 on the diagonal): two passes of the pair kernel, exact
 * (no difference quotient). Breakage (src/breakage_kernels.cuh:115-251) is
 * linear in N where its guard S != 0 && N > 2.2e-308 passes: its product is
 * the breakage RHS of v restricted to the bins whose N passes the guard. No
 * counterpart in the reference. */
int pbe_batch_jvp(pbe_batch_t plan, const double* N, const double* v,
                  const pbe_batch_cell_params_t* params, double* out, void* stream);

/* Linearly implicit integration of every cell: n_steps steps of size dt of
 * the two-stage Rosenbrock method ROS2 (second order, L-stable,
 * gamma = 1 + 1/sqrt(2)):
 *   (I - gamma dt J) k1 = rhs(N),  (I - gamma dt J) k2 = rhs(N + dt k1) - 2 k1,
 *   N += 3/2 dt k1 + 1/2 dt k2,  J = J(N) for both stages.
 * Each linear system is solved matrix-free by GMRES with krylov_dim
 * (1..64) Arnoldi steps and no restart, right-preconditioned by
 * 1 + gamma dt (death and breakage loss rate of bin i); every Arnoldi step
 * takes one pbe_batch_jvp. resid (device, n_cells, may be NULL) receives per
 * cell the largest relative least-squares residual of the call's solves
 * (0: solved exactly within round-off). Plan-owned memory grows on first use
 * by (krylov_dim + 8) packed vectors. The reference leaves time integration
 * to the caller (examples/common/pbe_examples_utils.hpp:391-456). */
int pbe_batch_ros2(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params, double dt,
                   int n_steps, int krylov_dim, double* resid, void* stream);

/* ROS2 to t_end with a step size per cell: the error of a step is the RMS of
 * dt (k1 + k2) / 2 -- its difference to the embedded first-order solution
 * N + dt k1 -- over atol + rtol max(|N|, |N_new|); a step is accepted when it
 * is <= 1, and the next dt is 0.9 err^(-1/2) dt clamped to [0.2, 5] dt (no
 * growth after a rejection, never past t_end). Solves as pbe_batch_ros2, with
 * gamma dt per cell. steps / rejects (host, n_cells) and *attempts as for
 * pbe_batch_rk45; returns cudaErrorNotReady (600) when some cell has not
 * reached t_end within max_attempts. */
int pbe_batch_ros2_adaptive(pbe_batch_t plan, double* N, const pbe_batch_cell_params_t* params,
                            double t_end, double rtol, double atol, double dt0, int krylov_dim,
                            int max_attempts, int* steps, int* rejects, int* attempts,
                            double* resid, void* stream);

/* Krylov tolerance of the plan's Rosenbrock solves (default 0): a cell's
 * GMRES ends once its least-squares residual |r - A x| <= tol |r|, before
 * krylov_dim steps; the cell is then left out of the remaining
 * Jacobian-vector products of that solve. 0 runs every solve for krylov_dim
 * steps (or to an exact breakdown). tol in [0, 1), else cudaErrorInvalidValue. */
int pbe_batch_set_krylov_tol(pbe_batch_t plan, double tol);

/* Restarts of the plan's Rosenbrock solves (default 0): a cell whose relative
 * residual after krylov_dim steps is above the Krylov tolerance runs another
 * cycle on r - A x, up to `restarts` more (each one Jacobian-vector product for
 * the residual plus up to krylov_dim steps; cells within the tolerance are
 * left out). With tol 0 every cell runs every cycle. The reported resid is
 * the residual after the cell's last cycle. restarts in [0, 1000], else
 * cudaErrorInvalidValue. */
int pbe_batch_set_krylov_restarts(pbe_batch_t plan, int restarts);

/* Mesh-field (structure-of-arrays) layout for CFD coupling: soa[i * ld + c]
 * (device) is bin i of cell c, one field per bin over the cells, ld >=
 * n_cells; rows i < n_c of every cell are read (from_soa: soa -> packed N)
 * or written (to_soa: packed N -> soa); entries beyond a cell's n_c are not
 * touched. A tiled transpose through shared memory, coalesced both ways. The
 * reference's README names this use (many cells of a CFD mesh) but ships no
 * layer for it. */
int pbe_batch_from_soa(pbe_batch_t plan, const double* soa, long long ld, double* N, void* stream);
int pbe_batch_to_soa(pbe_batch_t plan, const double* N, double* soa, long long ld, void* stream);

/* Schedule in use: group_size[c] (16 entries) = threads per tile task for
 * cells with floor(log2(n)) == c (0 where no cell falls), *n_bundles = the
 * number of bundles in the persistent launch. Either pointer may be NULL. */
int pbe_batch_schedule(pbe_batch_t plan, int* group_size, int* n_bundles);

/* ---------------------------------------------------------------------------
 * Checkpointed RK4 adjoint of one instance (no counterpart in the reference,
 * which has no derivatives). A tape runs n_steps classical RK4 steps of size
 * dt -- the stage arithmetic of the reference examples' rk4_step
 * (examples/common/pbe_examples_utils.hpp:416-456) -- saving N every
 * checkpoint_every steps; the backward pass recomputes one segment at a time
 * from its checkpoint and reverses every step with the VJP kernels, so memory
 * is (n_steps / checkpoint_every + 4 checkpoint_every + 16) n doubles.
 * Step s uses parameter set step_set[s] (step_set NULL: set 0) of agg_sets /
 * brk_sets (host arrays of n_sets structs; either may be NULL for a run
 * without that term; all sets share n, kernel_type, selection and n_quad).
 * ------------------------------------------------------------------------- */
typedef struct pbe_rk4_tape* pbe_rk4_tape_t;

int pbe_rk4_tape_create(pbe_rk4_tape_t* tape, int n_steps, double dt, int checkpoint_every,
                        int n_sets, const pbe_agg_params_t* agg_sets,
                        const pbe_brk_params_t* brk_sets, const int* step_set);

int pbe_rk4_tape_destroy(pbe_rk4_tape_t tape);

/* N (device, n): N(0) in, N(T) out. x, t_q, bw_q (device) are used again by
 * the backward pass and must stay valid until it is enqueued. */
int pbe_rk4_tape_forward(pbe_rk4_tape_t tape, double* N, const double* x, const double* t_q,
                         const double* bw_q, void* stream);

/* Given lambda_T = dL/dN(T) (device, n), writes gN0 = dL/dN(0) (device, n),
 * g_agg[3 m + j] = dL/d(beta0, beta_br, beta_sh)[j] of set m and
 * g_brk[4 m + j] = dL/d(S0, v_ref, alpha, v_min)[j] of set m (device; may be
 * NULL for an absent term). Returns cudaErrorInvalidValue before a forward. */
int pbe_rk4_tape_backward(pbe_rk4_tape_t tape, const double* lambda_T, double* gN0,
                          double* g_agg, double* g_brk, void* stream);

/* ---------------------------------------------------------------------------
 * Daughter tables for the breakage calls (host function, no GPU involved;
 * the reference documents the convention -- fragment volume t_q x_j, bw_q
 * fragments per event, include/pbe_cuda/breakage.cuh:43-50 -- but builds the
 * tables by hand in its examples and has no power-law table):
 *   PBE_DAUGHTER_SYMMETRIC  t = {1/2}, bw = {2}                      (1 entry)
 *   PBE_DAUGHTER_EROSION    t = {1 - param, param}, bw = {1, 1}      (2 entries)
 *   PBE_DAUGHTER_UNIFORM    Gauss-Legendre on (0, 1), bw = 2 w       (order entries)
 *   PBE_DAUGHTER_POWERLAW   b(v|v') = (p+2) v^p / v'^(p+1), p = param > -1:
 *                           Gauss-Legendre on (0, s) and (s, 1), s = param2
 *                           (0 means 1/2), bw = (p+2) t^p w     (2 order entries)
 * Writes at most `capacity` entries to t_q / bw_q (host arrays) and the count
 * to *n_quad; with t_q or bw_q NULL and capacity 0 it only reports the count.
 * Returns 0, or 1 (cudaErrorInvalidValue) for a bad kind, order, parameter or
 * a too small capacity. */
enum { PBE_DAUGHTER_SYMMETRIC = 0, PBE_DAUGHTER_EROSION = 1, PBE_DAUGHTER_UNIFORM = 2,
       PBE_DAUGHTER_POWERLAW = 3 };
int pbe_daughter_table(int kind, int order, double param, double param2, double* t_q,
                       double* bw_q, int capacity, int* n_quad);

/* Human-readable name of a return code (cudaGetErrorString). */
const char* pbe_error_string(int code);

/* Library version, e.g. 100 for 0.1.0. */
int pbe_version(void);

/* Diagnostic (no reference counterpart): on the current device, the bytes the
 * library's private scratch pool holds from the driver (*reserved_bytes) and
 * the high-water mark of its bytes in use (*used_high_bytes) since the pool
 * was created or the mark was last reset; reset_high != 0 resets the mark
 * after reading it. Both are 0 before the first pool-using call on the
 * device. Lets a caller check which calls take scratch from the pool. */
int pbe_scratch_pool_usage(unsigned long long* reserved_bytes,
                           unsigned long long* used_high_bytes, int reset_high);

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
