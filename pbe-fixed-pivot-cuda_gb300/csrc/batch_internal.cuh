// =============================================================================
// batch_internal.cuh -- device layouts and launchers of the batched-cell path
// (many independent PBE cells with uneven section counts in one launch).
//
// Cells reference grids. Every cell c uses the first n_c pivots of its grid
// g(c) (n_c <= n_g), so cells that share a grid also share the grid's per-bin
// values, per-lag tables and breakage fragment tables, which are built once
// per plan. Cell state is packed: cell c owns [off_c, off_c + n_c) of every
// per-bin array (N, rhs and the stage arrays), off = prefix sum of n in cell
// order.
// =============================================================================
#pragma once

#include "pbe_internal.cuh"
#include "pbe_gb300.h"

namespace pbe_gb300 {

struct BatchGridDev {
    int off;     // first bin in the packed grid arrays
    int n;       // pivots
    int D0;      // first lag with Ld[d] == d (written by the grid kernel)
    int geo;     // 1 when verified geometric (written by the grid kernel)
    int foff;    // first entry of the grid's run-start table (nq * (n + 2) ints)
    int woff;    // first entry of the grid's fragment weights (nq * n doubles)
    int pad0, pad1;
};

struct BatchCellDev {
    int off;       // first bin in the packed cell arrays
    int n;         // sections of the cell (<= its grid's n)
    int grid;
    int tile_off;  // first hand-over slot of the cell's tiles (tile t at tile_off + t)
};

// Device pointers of a plan: grid tables (static) and per-stage cell arrays.
struct BatchDev {
    BatchGridDev* grids;
    const BatchCellDev* cells;
    int n_grids, n_cells;
    int kernel;        // aggregation kernel type, -1 = no aggregation
    int selection;     // breakage selection, -1 = no breakage
    int nq;            // quadrature points (0 = no breakage)
    // breakage gather (in the padding after nq, so the struct keeps its size):
    // bit kBrkTasks: gathered from SN by the pair tasks in their epilogues
    // (their own bins) instead of by the prep kernel (one CTA per cell, into
    // Bk); plans of few cells take it, so that one large cell's prep does not
    // hold up the launch, while many cells balance the prep CTAs anyway.
    // bit kBrkNone: no breakage term in this pass (the second pass of a
    // Jacobian-vector product).
    int brk;
    // per grid bin (packed by BatchGridDev::off)
    double* gx; double* ga; double* gia; double* ginv_dx; double* gBd; double* gSd; int* gLd;
    double* gSl;    // shear factor of lag d seen from the larger member: (1 + rho)^3 x_0 / x_d
    // breakage fragment tables: bfirst[foff + q (n+2) + m + 1] = first j with
    // lo(q, j) >= m; bwlo / bwhi[woff + q n + j] = bw_q times the shares of the
    // fragment x_j t_q at lo and lo + 1 (all of bw_q at lo when clipped)
    int* bfirst; double* bwlo; double* bwhi;
    int* blo;       // bracket of fragment (q, j) (-1: below x[0]), same index as bwlo
    // per cell bin (packed by BatchCellDev::off), rewritten every stage
    double* Y;      // stage state (the RHS argument)
    double* Nj;     // j-side N factor: beta N (beta0, beta_br)
    double* Hj;     // j-side x N factor: beta x N (beta0, beta_sh)
    double* Hk;     // x N (Sum, Product)
    double* SN;     // S(x) N, 0 where the breakage guard skips the bin
    double* Bk;     // breakage term of the stage (gathered by the prep kernel, brk without kBrkTasks)
    double* k;      // stage derivative (RK4)
    double* kacc;   // k1 + 2 k2 + 2 k3 (+ k4)
    // Jacobian-vector passes (batch_jvp.cu): the j-side vector of the pass,
    // unscaled (null for an RHS evaluation), and x times it
    const double* A;
    double* Ha;
    double* mom;    // [n_cells * 8] moments of the stage state (death term), [5] clip sum
    int* counter;   // [8] task counter of the persistent kernel
    // hand-over of a tile's first bin (tiles aligned to the cell's top; tile t
    // owns bins [n - W (t+1), n - W t)): its own value, the carry of the tile
    // below, and a ticket that both bump once per launch (odd = second)
    double* tfirst; double* tcarry; int* tticket;   // [sum of the cells' tiles]
    // schedule
    const int4* bundles;   // {first task, tasks, group size, 0}
    const int4* tasks;     // {cell, first bin, lag chunk, chunks of the tile}
    // lag chunks of the tiles (plans with few tiles: see build_schedule):
    // chunk c of a tile covers the lags [c Cg, (c + 1) Cg); the tile's last
    // chunk task (a ticket that wraps to 0 with it: no reset needed) adds the
    // chunks' slot sums in order and runs the epilogue
    int Cg;                // lags per chunk (0: no chunks)
    int cbound;            // most chunks of a tile
    double* cpart;         // [tiles * cbound * 2 kTileW]
    unsigned* cticket;     // [tiles] lag-chunk tasks of the tile done (wraps at nct)
    int n_bundles;
    int num_sms;
    // [n_cells] or null: a cell with a nonzero entry is left out of the prep
    // and pair launches (its outputs keep their old values): the finished
    // cells of an adaptive run, the ended solves of a GMRES. The entries do not
    // change during a launch, so all tasks of a cell agree.
    const int* skip;
    // [total] or null: S(x_i) of every cell bin for the parameters of the
    // current call (an RHS, a Jacobian-vector product, RK4 steps, embedded
    // RK, Rosenbrock, the tape), computed once at its start by batch_sel;
    // null: the kernels evaluate the selection function per bin
    const double* Sx;
};
constexpr int kBrkTasks = 1;
constexpr int kBrkNone = 2;

// Scratch of the batched VJP (batch_vjp.cu).
struct BatchVjpDev {
    double* h;             // x N per cell bin
    double* D;             // lambda slopes per cell bin
    double* mom;           // [n_cells * 16]: moments of N (0..4) and of lambda N (5..9)
    double* tpart;         // [2 * tiles]: parameter partials per row tile
    const int* tile_off;   // [n_cells + 1]: first row-tile slot of each cell
    const int4* bundles;   // row-tile bundles {first task, tasks, group size, 0}
    const int4* tasks;     // {cell, first row, 0, 1}
    int n_bundles;
    int* counter;
};

// Stage modes of the per-cell prep kernel (RK4 as the reference examples
// write it, examples/common/pbe_examples_utils.hpp:409-456):
enum BatchStage : int {
    kStageRhs     = 0,  // Y = N as given (RHS evaluation, RK4 stage 1 of the first step)
    kStageNext    = 1,  // kacc += k4; N += dt/6 kacc; Y = N (stage 1 of a later step)
    kStageTwo     = 2,  // kacc = k1; Y = N + c k1
    kStageThree   = 3,  // kacc += 2 k; Y = N + c k (stages 3 and 4)
    kStageFinish  = 4,  // kacc += k4; N += dt/6 kacc (no RHS follows)
    kStageCombine = 5,  // Y = N + dt_c sum_j a_j k_j (embedded RK stages, per-cell dt)
};

// Stage combination of an explicit RK method with a per-cell step:
// Y = N + dt[c] (a[0] k[0] + ... + a[nk-1] k[nk-1]), summed in that order.
struct StageCombine {
    const double* k[7];    // packed stage derivatives
    double a[7];
    int nk;
    const double* dt;      // [n_cells]
};

// Per-cell step control of the embedded RK 5(4) integrator.
struct Rk45Ctl {
    double* t;             // [n_cells] time reached
    double* dt;            // [n_cells] next step (0 once done)
    int* status;           // [n_cells] 0 running, 1 reached t_end, 2 step underflow
    int* steps;            // [n_cells] accepted steps
    int* rejects;          // [n_cells] rejected steps
    int* done;             // [1] cells with status != 0
    double t_end, rtol, atol;
};

// GMRES(m) state of the batched Rosenbrock solves (batch_implicit.cu).
constexpr int kGmresMaxDim = 64;
struct GmresDev {
    double* V;       // [(m + 1) * total] Arnoldi vectors, packed like the cell state
    double* Z;       // [total] P^-1 v_j: the operand of the next Jacobian-vector product
    double* W;       // [total] J z on entry of an Arnoldi step, then its new direction
    double* P;       // [total] diagonal preconditioner
    double* H;       // [n_cells * (m + 1) * m] rotated Hessenberg columns (column-major)
    double* gv;      // [n_cells * (m + 1)] rotated right-hand side of the least squares
    double* cs;      // [n_cells * m] Givens rotations
    double* sn;
    double* beta0;   // [n_cells] |r|
    int* kval;       // [n_cells] Arnoldi steps taken
    int* done;       // [n_cells] solve ended (converged, breakdown or m steps)
    const double* gtc;   // [n_cells] gamma dt per cell (adaptive steps), or null: gt
    const int* skip;     // [n_cells] or null: cells whose solve is not run (x = 0)
    // restarted solves: a cell whose residual after a cycle of m steps is above
    // tol |r| starts another cycle on r - A x (up to `restarts` more)
    double* R;       // [total] residual r - A x of the current solution
    double* rnorm;   // [n_cells] |r| of the system (tol is relative to it)
    double* last;    // [n_cells] |r - A x| / |r| after the cell's last cycle
    int* conv;       // [n_cells] 1: no further cycle (within tol, r = 0, or skipped)
    long long total;
    int m;
    int restarts;
    double gt;       // gamma dt
    double tol;      // a solve ends once |r - A x| <= tol |r| (0: after m steps or breakdown)
};

// Launchers (batch_kernels.cu). All are asynchronous on `s`.
// Once per plan, before any launch (and outside stream capture): the
// persistent kernel's shared-memory attribute for `kernel`.
cudaError_t batch_kernel_setup(int kernel);
cudaError_t batch_grid_tables(const BatchDev& d, const double* t_q, const double* bw_q,
                              int max_grid_n, cudaStream_t s);
// Prep of a stage: state update per `stage`, stage arrays, moments, counter reset.
// N: state (read, and written by kStageNext / kStageFinish); Yrhs: the state
// the RHS is evaluated at (N itself for kStageRhs / kStageNext).
cudaError_t batch_prep(const BatchDev& d, double* N, const pbe_batch_cell_params_t* params,
                       int stage, double c, double dt6, cudaStream_t s);
// Prep of an embedded-RK stage: Y = N + dt_c sum_j a_j k_j, then as batch_prep.
cudaError_t batch_prep_combine(const BatchDev& d, double* N, const pbe_batch_cell_params_t* params,
                               const StageCombine& sc, cudaStream_t s);
// Error estimate, accept / reject and next step of every running cell (one
// CTA per cell): err = RMS over bins of dt sum_j e_j k_j / (atol + rtol
// max(|N|, |Y|)); accepted: N = Y, k[0] = k[6] (first stage of the next step).
cudaError_t batch_rk45_control(const BatchDev& d, double* N, const double* Y,
                               const StageCombine& err, double* k0, const Rk45Ctl& ctl,
                               cudaStream_t s);
// Mesh-field layout (batch_soa.cu): soa[i ld + c] <-> N[off_c + i] for the
// bins i < n_c of every cell (to_packed: soa -> N), max_n = the longest cell.
cudaError_t batch_soa(const BatchDev& d, const double* src, double* dst, long long ld, int max_n,
                      bool to_packed, cudaStream_t s);

// GMRES steps (batch_implicit.cu): start (preconditioner at N, v_0 = r/|r|),
// Arnoldi step j (after W = J(N) Z), finish (x = P^-1 V y, resid = relative
// least-squares residual per cell, may be null); elementwise helpers.
// first: the first cycle of a solve (records |r|, clears conv); later cycles
// run only the cells without conv. finish: acc adds to x (later cycles);
// final folds each cell's last relative residual into resid (max).
// restart: R = r - A x (W = J x on entry) for the cells without conv.
cudaError_t batch_gmres_restart(const BatchDev& d, const GmresDev& g, const double* r,
                                const double* x, cudaStream_t s);
cudaError_t batch_gmres_start(const BatchDev& d, const GmresDev& g, const double* N, const double* r,
                              const pbe_batch_cell_params_t* params, bool first, cudaStream_t s);
cudaError_t batch_gmres_arnoldi(const BatchDev& d, const GmresDev& g, int j, cudaStream_t s);
cudaError_t batch_gmres_finish(const BatchDev& d, const GmresDev& g, double* x, double* resid,
                               bool acc, bool final, cudaStream_t s);
cudaError_t batch_lincomb(double* out, double a, const double* X, double b, const double* Y,
                          long long total, int num_sms, cudaStream_t s);
cudaError_t batch_ros_update(double* N, double c1, const double* K1, double c2, const double* K2,
                             long long total, int num_sms, cudaStream_t s);
// Adaptive ROS2 (per-cell dt in ctl.dt, Rk45Ctl conventions): Y = N + dt_c K1
// and gtc[c] = gamma dt_c for every cell; then, after the second stage, the
// controller: err = RMS of dt_c (K1 + K2) / 2 (the difference to the embedded
// first-order solution N + dt_c K1) over atol + rtol max(|N|, |N_new|),
// accept when <= 1 (N = N + dt_c (3/2 K1 + 1/2 K2)), next dt from
// 0.9 err^(-1/2) clamped to [0.2, 5].
cudaError_t batch_ros2_stage(const BatchDev& d, const double* N, const double* K1, double* Y,
                             double* gtc, const Rk45Ctl& ctl, double gamma, cudaStream_t s);
cudaError_t batch_ros2_control(const BatchDev& d, double* N, const double* K1, const double* K2,
                               const Rk45Ctl& ctl, cudaStream_t s);

// Prep of one Jacobian-vector pass (batch_kernels.cu, batch_jvp_prep_kernel):
// j side from A, k side from B, breakage (brk) as the product of its Jacobian
// at the state G with B, else zero. Followed by batch_main with Y = B and a
// copy of d whose A = A.
// Sx[off_c + i] = S(x_i) of cell c's parameters, every bin of the plan
// (total = the packed length).
cudaError_t batch_sel(const BatchDev& d, const pbe_batch_cell_params_t* params, double* Sx,
                      long long total, cudaStream_t s);
cudaError_t batch_jvp_prep(const BatchDev& d, const double* A, const double* B, const double* G,
                           const pbe_batch_cell_params_t* params, bool brk, cudaStream_t s);
// Persistent RHS kernel over the plan's bundles: out (+)= RHS(Y) for every cell.
cudaError_t batch_main(const BatchDev& d, const double* Y, const pbe_batch_cell_params_t* params,
                       double* out, bool accumulate, cudaStream_t s);
// Same over an explicit bundle list (the autotuner's candidate schedules).
cudaError_t batch_main_bundles(const BatchDev& d, const double* Y,
                               const pbe_batch_cell_params_t* params, double* out,
                               bool accumulate, const int4* bundles, const int4* tasks,
                               int n_bundles, cudaStream_t s);
// Death term N_i sum_k beta(x_i, x_k) N_k of every cell (death_gemm.cu):
// method 0 = per-cell moments, 1 = FP64 tensor-core GEMM over the work items
// {grid, first row of gcells, rows <= 64, first bin} (cells grouped by grid).
// (DMMA: S > 1 k slices with partials in part [S * total], then a reduce;
// Bm: every grid's B at boff[g] (device; hboff the host copy), filled once per
// plan by batch_death_b for the grids in grids_used.)
cudaError_t batch_death_b(const BatchDev& d, const int* grids_used, int n_used, double* Bm,
                          const long long* hboff, cudaStream_t s);
cudaError_t batch_death(const BatchDev& d, const double* N, const pbe_batch_cell_params_t* params,
                        double* out, int method, const int4* items, int n_items,
                        const int* gcells, double* part, int S, long long total, const double* Bm,
                        const long long* boff, cudaStream_t s);
// Batched VJP: gN += dL/dN, gparams[8 c + j] += dL/d(parameter j of cell c)
// for L = lambda . RHS(N) (batch_vjp.cu). batch_vjp_setup once per plan.
cudaError_t batch_vjp_setup(int kernel);
cudaError_t batch_vjp(const BatchDev& d, const BatchVjpDev& vd, const double* N, const double* lam,
                      double* gN, double* gparams, const pbe_batch_cell_params_t* params,
                      cudaStream_t s);
// Adjoint stage helpers over n packed entries: a = w lp (+ c mu), mu = 0; lsum += mu.
cudaError_t batch_adj_coeff(double* a, const double* lp, double* mu, double w, double c,
                            long long n, bool first, cudaStream_t s);
cudaError_t batch_adj_sum(double* lsum, const double* mu, long long n, cudaStream_t s);
// Per-cell RK4 stage update for the per-cell launch loop (one cell, n bins).
cudaError_t cell_stage(double* N, const double* k, double* kacc, double* Y, int n, int stage,
                       double c, double dt6, cudaStream_t s);

} // namespace pbe_gb300
