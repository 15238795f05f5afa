// =============================================================================
// batch_kernels.cu -- batched-cell RHS and RK4 stage kernels (sm_103a, FP64).
//
// Per plan (once): batch_grid_kernel builds each grid's per-bin values, the
// beta-free per-lag tables and the geometric check; batch_frag_kernel builds
// the breakage fragment tables of each grid (brackets, weights, run starts).
//
// Per RHS evaluation (two launches):
//  * batch_prep_kernel, one CTA per cell: the RK4 stage update of the cell's
//    state, the stage arrays (j-side factors carrying the cell's kernel
//    coefficients, S(x) N for breakage), the five death moments and the sum
//    of the cell's clipped pairs.
//  * batch_main_kernel, persistent: CTAs pull "bundles" from an atomic
//    counter, largest first. A bundle holds 256/T tile tasks (cell, first bin)
//    that run side by side on groups of T threads; T is chosen per section
//    count class by the plan (autotuned or by rule), so a 64-section cell is
//    not spread over 256 threads. A task runs the shared tile body
//    (agg_tile.cuh), gathers the breakage term of its bins from S N (a few
//    fragments per bin and quadrature point), adds the prep kernel's clip sum
//    and writes its bins once: no atomics, and a fixed summation order for a
//    fixed schedule. The gather is spread over all tasks instead of one CTA
//    per cell, so a large cell's prep does not hold up the launch.
// =============================================================================
#include "batch_internal.cuh"
#include "agg_tile.cuh"

namespace pbe_gb300 {
namespace {

constexpr int W = kTileW;

// ---------------------------------------------------------------------------
// Grid tables: one CTA per grid. Per bin: a, 1/a, 1/dx; per lag d (= bin
// index): Bd = c_d * (1 or rho + 1/rho + 2), Sd = c_d (1 + rho)^3 with
// rho = (x_d / x_0)^(1/3), c_d = 1/2 for d = 0 (beta is applied per cell, on
// the j side); Ld = bracket of x_0 + x_d. Geometric check as the
// single-instance prep (max |ln(x_i/x_0) - i ln r| <= kGeoTol, x_1 <= 64 x_0).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
batch_grid_kernel(BatchDev d)
{
    __shared__ double sh[8];
    __shared__ int d0_s;
    BatchGridDev* gd = d.grids + blockIdx.x;
    const int n = gd->n;
    const double* x = d.gx + gd->off;
    if (threadIdx.x == 0) d0_s = n;
    __syncthreads();
    const bool brownian_like = (d.kernel >= 3);
    double dev = 0.0;
    int d0 = n;
    const double x0 = x[0];
    const double ax0 = cbrt(x0);
    const GeoFit fit = geo_fit(x0, x[n - 1], n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double xi = x[i];
        const double ai = cbrt(xi);
        d.ga[gd->off + i] = ai;
        d.gia[gd->off + i] = 1.0 / ai;
        d.ginv_dx[gd->off + i] = (i < n - 1) ? 1.0 / (x[i + 1] - xi) : 0.0;
        const double c = (i == 0) ? 0.5 : 1.0;
        const double rho = ai / ax0;
        const double s = 1.0 + rho;
        d.gBd[gd->off + i] = brownian_like ? c * (rho + 1.0 / rho + 2.0) : c;
        d.gSd[gd->off + i] = c * (s * s) * s;
        d.gSl[gd->off + i] = (s * s) * s * (x0 / xi);
        const double v = x0 + xi;
        const int L = (dbits(v) >= dbits(x[n - 1])) ? kLagClipAll : bracket_from(x, n, v, i);
        d.gLd[gd->off + i] = L;
        if (L == i) d0 = min(d0, i);
        if (n >= 2) {
            double e = geo_dev(fit, xi, i);
            if (!(e == e)) e = 1.0;
            dev = fmax(dev, e);
        }
    }
    atomicMin(&d0_s, d0);
    dev = warp_max(dev);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dev;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, sh[w]);
        const bool ratio_ok = n >= 2 && x[1] <= 64.0 * x[0];
        gd->geo = (n >= 2 && mx <= kGeoTol && ratio_ok) ? 1 : 0;
        gd->D0 = d0_s;
    }
}

// Breakage fragment tables: one CTA per grid, threads over (q, j). Fragment
// v = x_j t_q has the bracket lo = frag_bracket (-1: clipped to bin 0, n-1:
// clipped to bin n-1); its shares of bw_q are
// (bw_q/(x_{lo+1} - x_lo)) (x_{lo+1} - v) and (...) (v - x_lo), as the
// reference splits contrib (src/breakage_kernels.cuh:197-216).
__global__ void __launch_bounds__(256)
batch_frag_kernel(BatchDev d, const double* __restrict__ t_q, const double* __restrict__ bw_q)
{
    const BatchGridDev gd = d.grids[blockIdx.x];
    const int n = gd.n, nq = d.nq;
    const double* x = d.gx + gd.off;
    for (int idx = threadIdx.x; idx < n * nq; idx += blockDim.x) {
        const int q = idx / n, j = idx - q * n;
        const double tq = t_q[q], bw = bw_q[q];
        const double v = x[j] * tq;
        const int lo = frag_bracket(x, n, v);
        double wl = bw, wh = 0.0;
        if (lo >= 0 && lo < n - 1) {
            const double xl = x[lo], xh = x[lo + 1];
            const double qq = bw / (xh - xl);
            wl = qq * (xh - v);
            wh = qq * (v - xl);
        }
        d.bwlo[gd.woff + q * n + j] = wl;
        d.bwhi[gd.woff + q * n + j] = wh;
        d.blo[gd.woff + q * n + j] = lo;
        int* fq = d.bfirst + gd.foff + q * (n + 2);
        const int lo_prev = (j == 0) ? -2 : frag_bracket(x, n, x[j - 1] * tq);
        for (int m = max(lo_prev + 1, -1); m <= lo; ++m) fq[m + 1] = j;
        if (j == n - 1)
            for (int m = max(lo + 1, -1); m <= n; ++m) fq[m + 1] = n;
    }
}

// ---------------------------------------------------------------------------
// Stage prep: one CTA per cell.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double sel_value(int F, double v, double S0, double v_ref,
                                            double alpha, double v_min)
{
    switch (F) {
    case 0: return selection<0>(v, S0, v_ref, alpha, v_min);
    case 1: return selection<1>(v, S0, v_ref, alpha, v_min);
    case 2: return selection<2>(v, S0, v_ref, alpha, v_min);
    default: return selection<3>(v, S0, v_ref, alpha, v_min);
    }
}

// RK4 stage arithmetic of the reference examples (pbe_examples_utils.hpp:432-455)
// with every product and sum rounded separately, as the host code does:
// stage = N + (c dt) k, N_new = N + (dt/6) (((k1 + 2 k2) + 2 k3) + k4).
__device__ __forceinline__ double stage_update(int stage, double* N, const double* k, double* kacc,
                                               double* Y, int i, double c, double dt6)
{
    double y;
    if (stage == kStageRhs) {
        y = N[i];
    } else if (stage == kStageNext || stage == kStageFinish) {
        const double s = __dadd_rn(kacc[i], k[i]);
        y = __dadd_rn(N[i], __dmul_rn(dt6, s));
        N[i] = y;
    } else {
        const double ki = k[i];
        kacc[i] = (stage == kStageTwo) ? ki : __dadd_rn(kacc[i], __dmul_rn(2.0, ki));
        y = __dadd_rn(N[i], __dmul_rn(c, ki));
        Y[i] = y;
    }
    return y;
}

// Per-cell stage update of the per-cell launch loop (same arithmetic).
__global__ void __launch_bounds__(256)
cell_stage_kernel(double* N, const double* k, double* kacc, double* Y, int n, int stage,
                  double c, double dt6)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) stage_update(stage, N, k, kacc, Y, i, c, dt6);
}

// Selection function of every cell bin for the given parameters: one thread
// per packed bin over the whole plan (its cell found by bisection of the
// cells' offsets), so that a large cell's transcendentals spread over all
// SMs instead of one CTA's; evaluated once per call instead of per stage.
__global__ void __launch_bounds__(256)
batch_sel_kernel(BatchDev d, const pbe_batch_cell_params_t* __restrict__ params,
                 double* __restrict__ Sx, long long total)
{
    for (long long e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
        int lo = 0, hi = d.n_cells;          // cells[lo].off <= e < cells[hi].off
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (d.cells[mid].off <= e) lo = mid; else hi = mid;
        }
        const BatchCellDev cd = d.cells[lo];
        const pbe_batch_cell_params_t P = params[lo];
        const double* x = d.gx + d.grids[cd.grid].off;
        Sx[e] = sel_value(d.selection, x[e - cd.off], P.S0, P.v_ref, P.alpha, P.v_min);
    }
}

// ---------------------------------------------------------------------------
// Clipped pairs of a cell (v >= x[n-1], all deposited on bin n-1), summed by
// the group of the task that owns bin n-1: per lag on a geometric grid (the
// pairs j in [n-1-Ld, n-1-d]), per row otherwise.
// ---------------------------------------------------------------------------
template <int K>
__device__ double cell_clip(const AggCellView& v, const TileGroup& G)
{
    const int n = v.n;
    double acc = 0.0;
    if (v.geo) {
        for (int d = G.lane; d < n; d += G.T) {
            const int L = v.Ld[d];
            const int jhi = n - 1 - d;
            const int jlo = (L >= kLagClipAll) ? 0 : max(0, n - 1 - L);
            const double B = v.Bd[d], S = v.Sd[d];
            for (int j = jlo; j <= jhi; ++j) {
                const double hj = NeedH<K>::j ? v.Hj[j] : 0.0;
                const double hk = NeedH<K>::k ? v.Hk[j + d] : 0.0;
                acc += rate_geo<K>(B, S, v.Nj[j], hj, v.Nk[j + d], hk);
            }
        }
    } else {
        const long long tb = dbits(v.x[n - 1]);
        for (int j = G.lane; j < n; j += G.T) {
            const double xj = v.x[j];
            int lo = j, hi = n - 1;   // xj + x[n-1] >= x[n-1] always holds
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (dbits(xj + v.x[mid]) >= tb) hi = mid; else lo = mid + 1;
            }
            const double Nj = v.Aj[j], hj = v.AHj[j], aj = v.a[j], iaj = v.ia[j];
            for (int k = lo; k < n; ++k)
                acc += rate_gen<K>(j == k, v.b0, v.bbr, v.bsh, Nj, hj, aj, iaj, v.Nk[k], v.Hk[k],
                                   v.a[k], v.ia[k]);
        }
    }
    return acc;
}

// One lane's part of the breakage gather of bin i (0 <= i < n) of a cell:
// quadrature points q = q0, q0 + nqp, ..., each adding the hi-shares of the
// fragments bracketed at i-1 and the lo-shares of those at i (bin 0 also the
// fragments clipped below x[0]). The nqp lanes of a bin then add their parts
// in a fixed butterfly.
__device__ __forceinline__ double brk_lane(const BatchDev& d, const BatchGridDev& gd,
                                           const double* SN, int n, int i, int q0, int nqp)
{
    const int ng = gd.n;
    double acc = 0.0;
    for (int q = q0; q < d.nq; q += nqp) {
        const int* fq = d.bfirst + gd.foff + q * (ng + 2);
        const double* wl = d.bwlo + gd.woff + q * ng;
        const double* wh = d.bwhi + gd.woff + q * ng;
        const int fa = min(max(fq[i], 0), n);         // first j with lo >= i-1
        const int fb = min(max(fq[i + 1], fa), n);    // first j with lo >= i
        const int fc = min(max(fq[i + 2], fb), n);    // first j with lo >= i+1
        if (i == 0) { for (int j = 0; j < fb; ++j) acc = fma(SN[j], wl[j], acc); }
        else        { for (int j = fa; j < fb; ++j) acc = fma(SN[j], wh[j], acc); }
        for (int j = fb; j < fc; ++j) acc = fma(SN[j], wl[j], acc);
    }
    return acc;
}

__device__ __forceinline__ int brk_lanes(int nq)
{
    int nqp = 1;
    while (nqp < nq && nqp < 32) nqp <<= 1;
    return nqp;
}

// Breakage term of every bin of a cell (one CTA; the prep kernels without
// kBrkTasks), minus S_i N_i: a warp covers 32/nqp bins, nqp = the quadrature
// points rounded up to a power of two (<= 32) lanes per bin.
__device__ void cell_breakage(const BatchDev& d, const BatchGridDev& gd, const double* SN,
                              double* Bk, int n)
{
    const int nqp = brk_lanes(d.nq);
    const int per_warp = 32 / nqp;
    const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int base = w * per_warp; base < n; base += nw * per_warp) {   // uniform per warp
        const int i = base + l / nqp;
        double acc = (i < n) ? brk_lane(d, gd, SN, n, i, l % nqp, nqp) : 0.0;
        for (int o = nqp >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (i < n && (l % nqp) == 0) Bk[i] = acc - SN[i];
    }
}

// The same term for the bins I .. I+W-1 of a cell (those in [0, n)), by a
// task's group into out[0 .. W) (kBrkTasks): the same lanes per bin, loops and
// butterfly, so the sums are bitwise those of cell_breakage.
__device__ void tile_breakage(const BatchDev& d, const BatchGridDev& gd, const double* SN, int n,
                              int I, double* out, const TileGroup& G)
{
    const int nqp = brk_lanes(d.nq);
    const int per_warp = 32 / nqp;
    const int nw = G.T >> 5, w = G.lane >> 5, l = G.lane & 31;
    for (int base = w * per_warp; base < W; base += nw * per_warp) {   // uniform per warp
        const int t = base + l / nqp;
        const int i = I + t;
        const bool in = t < W && i >= 0 && i < n;
        double acc = in ? brk_lane(d, gd, SN, n, i, l % nqp, nqp) : 0.0;
        for (int o = nqp >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (t < W && (l % nqp) == 0) out[t] = in ? acc - SN[i] : 0.0;
    }
}

// ---------------------------------------------------------------------------
// Stage prep: one CTA per cell. Pass 1 (per bin): the stage update, the stage
// arrays (S N for the breakage gather of the pair tasks) and the moment
// partials. Pass 2 (after a block barrier, so the whole cell's arrays are
// visible): the moments and the cell's clipped-pair sum (mom[5]).
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
batch_prep_kernel(BatchDev d, double* N, const pbe_batch_cell_params_t* __restrict__ params,
                  int stage, double c, double dt6, StageCombine sc)
{
    __shared__ double sh[8];
    if (d.skip && d.skip[blockIdx.x]) return;       // whole block
    const BatchCellDev cd = d.cells[blockIdx.x];
    const BatchGridDev gd = d.grids[cd.grid];
    const pbe_batch_cell_params_t P = params[blockIdx.x];
    const bool agg = d.kernel >= 0;
    const int F = d.selection;
    const int off = cd.off, n = cd.n;
    double* Nc = N + off;
    double* kc = d.k + off;
    double* ac = d.kacc + off;
    double* Yc = d.Y + off;
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    // j-side coefficients: Nj = cN * N, Hj = cH * x N
    const double cN = (K <= 2) ? P.beta0 : P.beta_br;
    const double cH = (K == 1 || K == 2) ? P.beta0 : P.beta_sh;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const double dtc = (stage == kStageCombine) ? sc.dt[blockIdx.x] : 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double y;
        if (stage == kStageCombine) {
            double s_ = 0.0;
            for (int j = 0; j < sc.nk; ++j) s_ = fma(sc.a[j], sc.k[j][off + i], s_);
            y = fma(dtc, s_, Nc[i]);
            Yc[i] = y;
        } else {
            y = stage_update(stage, Nc, kc, ac, Yc, i, c, dt6);
        }
        if (stage == kStageFinish) continue;
        const double xi = x[i];
        const double h = xi * y;
        if (agg) {
            if (K != 2 && K != 4) d.Nj[off + i] = cN * y;
            if (NeedH<K>::j) d.Hj[off + i] = cH * h;
            if (NeedH<K>::k) d.Hk[off + i] = h;
            m[0] = fma(ia[i], y, m[0]);
            m[1] += y;
            m[2] = fma(a[i], y, m[2]);
            m[3] = fma(a[i] * a[i], y, m[3]);
            m[4] += h;
        }
        if (F >= 0) {
            const double S = d.Sx ? d.Sx[off + i] : sel_value(F, xi, P.S0, P.v_ref, P.alpha, P.v_min);
            d.SN[off + i] = (S != 0.0 && y > kBreakageNMin) ? S * y : 0.0;
        }
    }
    if (stage == kStageFinish) return;
    __syncthreads();                       // the cell's stage arrays are complete
    if (agg) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const double s = block_sum(m[q], sh);
            if (threadIdx.x == 0) d.mom[blockIdx.x * 8 + q] = s;
        }
        AggCellView v;
        v.x = x;
        v.Nk = (stage == kStageRhs || stage == kStageNext) ? Nc : Yc;
        v.Hk = d.Hk + off;
        v.Aj = v.Nk;
        v.AHj = v.Hk;
        v.Nj = d.Nj + off;
        v.Hj = d.Hj + off;
        v.Fs = v.Nk;
        v.a = a; v.ia = ia; v.inv_dx = d.ginv_dx + gd.off;
        v.Bd = d.gBd + gd.off; v.Sd = d.gSd + gd.off; v.Ld = d.gLd + gd.off;
        v.n = n; v.D0 = gd.D0; v.geo = gd.geo != 0;
        v.b0 = P.beta0; v.bbr = P.beta_br; v.bsh = P.beta_sh;
        const TileGroup G{0, static_cast<int>(threadIdx.x), static_cast<int>(blockDim.x)};
        const double clip = block_sum(cell_clip<K>(v, G), sh);
        if (threadIdx.x == 0) d.mom[blockIdx.x * 8 + 5] = clip;
    }
    if (d.nq > 0 && !(d.brk & kBrkTasks)) cell_breakage(d, gd, d.SN + off, d.Bk + off, n);
}

// Hand-over of bin `bin` of a cell (the first bin of tile slot `slot`): its
// owner tile and the tile below each store their part and bump the ticket;
// the second (odd count: each launch adds two) writes own + carry. The sum of
// two is the same whichever is second. Called by one thread.
__device__ __forceinline__ void batch_first_done(const BatchDev& d, double* out, bool accumulate,
                                                 int bin, int slot)
{
    __threadfence();
    if ((atomicAdd(d.tticket + slot, 1) & 1) == 0) return;
    __threadfence();
    const double v = __ldcg(d.tfirst + slot) + __ldcg(d.tcarry + slot);
    double* o = out + bin;
    *o = accumulate ? __ldcg(o) + v : v;
}

// ---------------------------------------------------------------------------
// Prep of one Jacobian-vector pass (one CTA per cell). The aggregation RHS is
// quadratic: R(N) = T(N, N) with T(a, b) = sum over pairs j <= k of
// c_d beta(j, k) a_j b_k (deposits as the RHS; death b_i sum_k beta_ik a_k),
// so J(N) v = T(N, v) + T(v, N), two passes of the persistent pair kernel
// with the j side from a and the k side from b. This prep builds the j-side
// arrays from a (coefficient-scaled, and unscaled for the generic path), the
// k-side x b, the moments of a (death b_i sum_k beta_ik a_k), the clipped
// pairs' sum of T(a, b), and the breakage input: the breakage RHS is linear
// in N wherever its guard passes, so with brk its Jacobian-vector product
// deposits S_j b_j as the RHS deposits S_j N_j, for the bins whose G_j (the
// state) passes the guard S_j != 0 && G_j > 2.2e-308 (SN = S b there, 0
// elsewhere; gathered here or by the pair tasks, as for the RHS); the pass
// without brk runs its pair kernel with kBrkNone.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256)
batch_jvp_prep_kernel(BatchDev d, const double* __restrict__ A, const double* __restrict__ Bv,
                      const double* __restrict__ Gs, const pbe_batch_cell_params_t* __restrict__ params,
                      int brk)
{
    __shared__ double sh[8];
    if (d.skip && d.skip[blockIdx.x]) return;       // whole block
    const BatchCellDev cd = d.cells[blockIdx.x];
    const BatchGridDev gd = d.grids[cd.grid];
    const pbe_batch_cell_params_t P = params[blockIdx.x];
    const bool agg = d.kernel >= 0;
    const int F = d.selection;
    const int off = cd.off, n = cd.n;
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const double cN = (K <= 2) ? P.beta0 : P.beta_br;
    const double cH = (K == 1 || K == 2) ? P.beta0 : P.beta_sh;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double ya = A[off + i], yb = Bv[off + i];
        const double xi = x[i];
        if (agg) {
            const double ha = xi * ya;
            if (K != 2 && K != 4) d.Nj[off + i] = cN * ya;
            if (NeedH<K>::j) d.Hj[off + i] = cH * ha;
            d.Ha[off + i] = ha;
            d.Hk[off + i] = xi * yb;
            m[0] = fma(ia[i], ya, m[0]);
            m[1] += ya;
            m[2] = fma(a[i], ya, m[2]);
            m[3] = fma(a[i] * a[i], ya, m[3]);
            m[4] += ha;
        }
        if (F >= 0) {
            double sn = 0.0;
            if (brk) {
                const double S = d.Sx ? d.Sx[off + i]
                                      : sel_value(F, xi, P.S0, P.v_ref, P.alpha, P.v_min);
                sn = (S != 0.0 && Gs[off + i] > kBreakageNMin) ? S * yb : 0.0;
            }
            d.SN[off + i] = sn;
        }
    }
    __syncthreads();                       // the cell's pass arrays are complete
    if (agg) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const double s_ = block_sum(m[q], sh);
            if (threadIdx.x == 0) d.mom[blockIdx.x * 8 + q] = s_;
        }
        AggCellView v;
        v.x = x;
        v.Nk = Bv + off;
        v.Hk = d.Hk + off;
        v.Nj = d.Nj + off;
        v.Hj = d.Hj + off;
        v.Aj = A + off;
        v.AHj = d.Ha + off;
        v.Fs = v.Nk;
        v.a = a; v.ia = ia; v.inv_dx = d.ginv_dx + gd.off;
        v.Bd = d.gBd + gd.off; v.Sd = d.gSd + gd.off; v.Ld = d.gLd + gd.off;
        v.n = n; v.D0 = gd.D0; v.geo = gd.geo != 0;
        v.b0 = P.beta0; v.bbr = P.beta_br; v.bsh = P.beta_sh;
        const TileGroup G{0, static_cast<int>(threadIdx.x), static_cast<int>(blockDim.x)};
        const double clip = block_sum(cell_clip<K>(v, G), sh);
        if (threadIdx.x == 0) d.mom[blockIdx.x * 8 + 5] = clip;
    }
    // first pass only (the second runs with kBrkNone)
    if (d.nq > 0 && !(d.brk & kBrkTasks) && brk) cell_breakage(d, gd, d.SN + off, d.Bk + off, n);
}

template <int K>
__device__ void batch_task(const BatchDev& d, const double* __restrict__ Yg,
                           const pbe_batch_cell_params_t* __restrict__ params, double* out,
                           bool accumulate, int4 tk, double* red, TileShared& sm,
                           const TileGroup& G)
{
    const int c = tk.x, I = tk.y, chunk = tk.z, nct = tk.w;
    if (d.skip && d.skip[c]) return;                // the whole group
    const BatchCellDev cd = d.cells[c];
    const BatchGridDev gd = d.grids[cd.grid];
    const int n = cd.n;
    const bool agg = d.kernel >= 0;
    AggCellView v;
    v.x = d.gx + gd.off;
    v.Nk = Yg + cd.off;
    v.Hk = d.Hk + cd.off;
    v.Aj = d.A ? d.A + cd.off : v.Nk;        // a Jacobian-vector pass: the j-side vector
    v.AHj = d.A ? d.Ha + cd.off : v.Hk;
    v.Nj = d.Nj + cd.off;
    v.Hj = d.Hj + cd.off;
    v.Fs = (K == 2) ? v.Hk : v.Nk;
    v.a = d.ga + gd.off; v.ia = d.gia + gd.off; v.inv_dx = d.ginv_dx + gd.off;
    v.Bd = d.gBd + gd.off; v.Sd = d.gSd + gd.off; v.Ld = d.gLd + gd.off;
    v.n = n;
    v.D0 = gd.D0;
    v.geo = gd.geo != 0;
    const pbe_batch_cell_params_t P = params[c];
    v.b0 = P.beta0; v.bbr = P.beta_br; v.bsh = P.beta_sh;
    // values the epilogue needs go through shared memory, so that they hold no
    // registers during the pair loop (read back after it)
    if (G.lane < 8) {
        const int l = G.lane;
        sm.cinfo[G.g][l] = (l < 5) ? d.mom[c * 8 + l]
                                   : (l == 5 ? P.beta0 : (l == 6 ? P.beta_br : P.beta_sh));
    }

    // tiles are aligned to the cell's top: I = n - W (tile + 1), I > -W
    const int tile = (n - I) / W - 1;
    const int St = -ilogb(v.x[max(I, 0)]);
    if (agg) {
        const int d_begin = nct > 1 ? chunk * d.Cg : 0;
        const int d_end = nct > 1 ? min(n, d_begin + d.Cg) : n;
        agg_tile_accumulate<K, true>(v, I, d_begin, d_end, St, red, sm, G);   // syncs the group first
        if (nct > 1) {
            // this chunk's slot sums; the tile's last chunk task adds all of
            // them in chunk order and runs the epilogue (nobody waits)
            constexpr int R2 = TileSlots<true>::rows;
            const int slot = cd.tile_off + tile;
            double* cp = d.cpart + static_cast<size_t>(slot) * d.cbound * R2;
            if (G.lane < R2) cp[chunk * R2 + G.lane] = sm.fin[G.g][G.lane];
            G.sync();
            if (G.lane == 0) {
                __threadfence();
                // the ticket counts 0 .. nct-1 and wraps to 0 on the last chunk
                // task, so it is ready for the next launch without a reset
                sm.last[G.g] = atomicInc(d.cticket + slot, static_cast<unsigned>(nct - 1))
                               == static_cast<unsigned>(nct - 1);
            }
            G.sync();
            if (!sm.last[G.g]) return;
            __threadfence();
            if (G.lane < R2) {
                double acc = 0.0;
                for (int q = 0; q < nct; ++q) acc += __ldcg(cp + q * R2 + G.lane);
                sm.fin[G.g][G.lane] = acc;
            }
            G.sync();
        }
#pragma unroll
        for (int q = 0; q < 5; ++q) v.M[q] = sm.cinfo[G.g][q];
        v.b0 = sm.cinfo[G.g][5]; v.bbr = sm.cinfo[G.g][6]; v.bsh = sm.cinfo[G.g][7];
    }
    const bool brk = d.nq > 0 && !(d.brk & kBrkNone);
    const bool brk_tasks = (d.brk & kBrkTasks) != 0;
    if (brk && brk_tasks) {
        tile_breakage(d, gd, d.SN + cd.off, n, I, sm.extra[G.g], G);
        G.sync();
    }
    if (G.lane < W) {
        const int i = I + G.lane;
        if (i >= 0) {
            double val = 0.0;
            if (agg) {
                double birth = agg_tile_birth<true>(v, I, G.lane, St, sm.fin[G.g]);
                if (i == n - 1) birth += d.mom[c * 8 + 5];     // clipped pairs (prep)
                val = birth - agg_death<K>(v, i);
            }
            if (brk) val += brk_tasks ? sm.extra[G.g][G.lane] : d.Bk[cd.off + i];   // breakage
            if (agg && G.lane == 0 && I >= 1) {
                // the w-part of slot I-1 comes from the tile below
                d.tfirst[cd.tile_off + tile] = val;
                batch_first_done(d, out, accumulate, cd.off + I, cd.tile_off + tile);
            } else {
                double* o = out + cd.off + i;
                *o = accumulate ? *o + val : val;
            }
        }
    } else if (agg && G.lane == W && tile >= 1) {
        // carry into bin I+W, the first bin of the tile above
        d.tcarry[cd.tile_off + tile - 1] = agg_tile_carry(v, I, St, sm.fin[G.g]);
        batch_first_done(d, out, accumulate, cd.off + I + W, cd.tile_off + tile - 1);
    }
}

#ifndef PBE_BATCH_CTAS
#define PBE_BATCH_CTAS 2
#endif
template <int K>
__global__ void __launch_bounds__(kMainThreads, PBE_BATCH_CTAS)
batch_main_kernel(BatchDev d, const double* __restrict__ Y,
                  const pbe_batch_cell_params_t* __restrict__ params, double* out, int accumulate,
                  const int4* __restrict__ bundles, const int4* __restrict__ tasks, int n_bundles)
{
    extern __shared__ double red[];     // [2 W][kMainThreads]
    __shared__ TileShared sm;
    __shared__ int s_b;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_b = atomicAdd(d.counter, 1);
        __syncthreads();
        const int b = s_b;
        __syncthreads();
        if (b >= n_bundles) break;
        const int4 bu = bundles[b];     // {first task, tasks, group size, 0}
        const int T = bu.z;
        const int g = tid / T;
        if (g < bu.y) {
            const TileGroup G{g, tid - g * T, T};
            batch_task<K>(d, Y, params, out, accumulate != 0, tasks[bu.x + g], red + g * T, sm, G);
        }
        __syncthreads();
    }
}

template <int K>
cudaError_t main_k(const BatchDev& d, const double* Y, const pbe_batch_cell_params_t* params,
                   double* out, bool accumulate, const int4* bundles, const int4* tasks,
                   int n_bundles, cudaStream_t s)
{
    const size_t smem = sizeof(double) * TileSlots<true>::rows * kMainThreads;
    cudaError_t e = cudaMemsetAsync(d.counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    if (n_bundles <= 0) return cudaSuccess;
    const int grid = n_bundles < PBE_BATCH_CTAS * d.num_sms ? n_bundles : PBE_BATCH_CTAS * d.num_sms;
    batch_main_kernel<K><<<grid, kMainThreads, smem, s>>>(d, Y, params, out, accumulate ? 1 : 0,
                                                          bundles, tasks, n_bundles);
    return cudaGetLastError();
}

template <int K>
cudaError_t attr_k()
{
    return cudaFuncSetAttribute(batch_main_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(sizeof(double) * TileSlots<true>::rows * kMainThreads));
}

} // namespace

cudaError_t batch_kernel_setup(int kernel)
{
    switch (kernel < 0 ? 0 : kernel) {
    case 0: return attr_k<0>();
    case 1: return attr_k<1>();
    case 2: return attr_k<2>();
    case 3: return attr_k<3>();
    case 4: return attr_k<4>();
    case 5: return attr_k<5>();
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_grid_tables(const BatchDev& d, const double* t_q, const double* bw_q,
                              int max_grid_n, cudaStream_t s)
{
    (void)max_grid_n;
    if (d.n_grids <= 0) return cudaErrorInvalidValue;
    batch_grid_kernel<<<d.n_grids, 256, 0, s>>>(d);
    if (d.nq > 0) batch_frag_kernel<<<d.n_grids, 256, 0, s>>>(d, t_q, bw_q);
    return cudaGetLastError();
}

namespace {
cudaError_t prep_any(const BatchDev& d, double* N, const pbe_batch_cell_params_t* params, int stage,
                     double c, double dt6, const StageCombine& sc, cudaStream_t s)
{
    if (d.n_cells <= 0) return cudaErrorInvalidValue;
    switch (d.kernel < 0 ? 0 : d.kernel) {
    case 0: batch_prep_kernel<0><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    case 1: batch_prep_kernel<1><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    case 2: batch_prep_kernel<2><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    case 3: batch_prep_kernel<3><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    case 4: batch_prep_kernel<4><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    case 5: batch_prep_kernel<5><<<d.n_cells, 256, 0, s>>>(d, N, params, stage, c, dt6, sc); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int K>
cudaError_t jvp_prep_k(const BatchDev& d, const double* A, const double* B, const double* G,
                       const pbe_batch_cell_params_t* params, bool brk, cudaStream_t s)
{
    batch_jvp_prep_kernel<K><<<d.n_cells, 256, 0, s>>>(d, A, B, G, params, brk ? 1 : 0);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256)
rk45_control_kernel(BatchDev d, double* N, const double* __restrict__ Y, StageCombine e,
                    double* k0, Rk45Ctl ctl)
{
    __shared__ double sh[8];
    __shared__ int accept_s;
    const int c = blockIdx.x;
    if (ctl.status[c] != 0) return;                 // whole block
    const BatchCellDev cd = d.cells[c];
    const int off = cd.off, n = cd.n;
    const double dt = ctl.dt[c];
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s_ = 0.0;
        for (int j = 0; j < e.nk; ++j) s_ = fma(e.a[j], e.k[j][off + i], s_);
        const double sc = ctl.atol + ctl.rtol * fmax(fabs(N[off + i]), fabs(Y[off + i]));
        const double r = (dt * s_) / sc;
        s2 = fma(r, r, s2);
    }
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        const double err = sqrt(s2 / n);
        const bool finite = (err == err) && err <= 1.7e308;
        const bool accept = finite && err <= 1.0;
        double fac;
        if (!finite) fac = 0.2;
        else if (err == 0.0) fac = 5.0;
        else fac = fmin(5.0, fmax(0.2, 0.9 * pow(err, -0.2)));
        if (!accept) fac = fmin(fac, 1.0);
        double t = ctl.t[c];
        if (accept) { t += dt; ctl.t[c] = t; ctl.steps[c] += 1; }
        else ctl.rejects[c] += 1;
        const double rem = ctl.t_end - t;
        double nd = fmin(dt * fac, rem);
        int st = 0;
        if (accept && rem <= 1e-12 * fmax(fabs(ctl.t_end), 1.0)) { st = 1; nd = 0.0; }
        else if (nd <= 1e-14 * fmax(fabs(ctl.t_end), 1.0)) { st = 2; nd = 0.0; }
        ctl.dt[c] = nd;
        if (st != 0) { ctl.status[c] = st; atomicAdd(ctl.done, 1); }
        accept_s = accept ? 1 : 0;
    }
    __syncthreads();
    if (accept_s) {
        const double* k6 = e.k[6];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            N[off + i] = Y[off + i];
            k0[off + i] = k6[off + i];     // first stage of the next step (FSAL)
        }
    }
}
} // namespace

cudaError_t batch_prep(const BatchDev& d, double* N, const pbe_batch_cell_params_t* params,
                       int stage, double c, double dt6, cudaStream_t s)
{
    const StageCombine none{};
    return prep_any(d, N, params, stage, c, dt6, none, s);
}

cudaError_t batch_sel(const BatchDev& d, const pbe_batch_cell_params_t* params, double* Sx,
                      long long total, cudaStream_t s)
{
    if (d.n_cells <= 0 || d.selection < 0 || total <= 0) return cudaErrorInvalidValue;
    const long long b = (total + 255) / 256, cap = 16LL * (d.num_sms > 0 ? d.num_sms : 1);
    batch_sel_kernel<<<static_cast<int>(b < cap ? b : cap), 256, 0, s>>>(d, params, Sx, total);
    return cudaGetLastError();
}

cudaError_t batch_jvp_prep(const BatchDev& d, const double* A, const double* B, const double* G,
                          const pbe_batch_cell_params_t* params, bool brk, cudaStream_t s)
{
    if (d.n_cells <= 0) return cudaErrorInvalidValue;
    switch (d.kernel < 0 ? 0 : d.kernel) {
    case 0: return jvp_prep_k<0>(d, A, B, G, params, brk, s);
    case 1: return jvp_prep_k<1>(d, A, B, G, params, brk, s);
    case 2: return jvp_prep_k<2>(d, A, B, G, params, brk, s);
    case 3: return jvp_prep_k<3>(d, A, B, G, params, brk, s);
    case 4: return jvp_prep_k<4>(d, A, B, G, params, brk, s);
    case 5: return jvp_prep_k<5>(d, A, B, G, params, brk, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_prep_combine(const BatchDev& d, double* N, const pbe_batch_cell_params_t* params,
                               const StageCombine& sc, cudaStream_t s)
{
    return prep_any(d, N, params, kStageCombine, 0.0, 0.0, sc, s);
}

cudaError_t batch_rk45_control(const BatchDev& d, double* N, const double* Y,
                               const StageCombine& err, double* k0, const Rk45Ctl& ctl,
                               cudaStream_t s)
{
    rk45_control_kernel<<<d.n_cells, 256, 0, s>>>(d, N, Y, err, k0, ctl);
    return cudaGetLastError();
}

cudaError_t batch_main_bundles(const BatchDev& d, const double* Y,
                               const pbe_batch_cell_params_t* params, double* out,
                               bool accumulate, const int4* bundles, const int4* tasks,
                               int n_bundles, cudaStream_t s)
{
    switch (d.kernel < 0 ? 0 : d.kernel) {
    case 0: return main_k<0>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    case 1: return main_k<1>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    case 2: return main_k<2>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    case 3: return main_k<3>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    case 4: return main_k<4>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    case 5: return main_k<5>(d, Y, params, out, accumulate, bundles, tasks, n_bundles, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_main(const BatchDev& d, const double* Y, const pbe_batch_cell_params_t* params,
                       double* out, bool accumulate, cudaStream_t s)
{
    return batch_main_bundles(d, Y, params, out, accumulate, d.bundles, d.tasks, d.n_bundles, s);
}

cudaError_t cell_stage(double* N, const double* k, double* kacc, double* Y, int n, int stage,
                       double c, double dt6, cudaStream_t s)
{
    if (n <= 0) return cudaErrorInvalidValue;
    cell_stage_kernel<<<(n + 255) / 256, 256, 0, s>>>(N, k, kacc, Y, n, stage, c, dt6);
    return cudaGetLastError();
}

} // namespace pbe_gb300
