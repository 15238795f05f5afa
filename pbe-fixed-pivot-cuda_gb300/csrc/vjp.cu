// =============================================================================
// vjp.cu -- vector-Jacobian products (adjoints) of the aggregation and
// breakage RHS, FP64, sm_103a. No counterpart in the reference.
//
// Given lambda = dL/drhs, the calls ADD dL/dN into gN and dL/d(parameters)
// into a small device array, like the forward calls add into rhs.
//
// Aggregation. For pair p = (j <= k): rate_p = c_p beta_jk N_j N_k (c = 1/2 on
// the diagonal), L = sum_p rate_p G_p with G_p = P_p - lambda_j - lambda_k,
// P_p = lambda_lo + w (lambda_hi - lambda_lo) (lambda_{n-1} for pairs clipped
// at x[n-1]). Then
//   dL/dN_m  = sum_k G(m,k) beta(m,k) N_k           (all partners k, k = m once)
//   dL/dbeta_X = 1/2 sum_m N_m A_X[m],  A_X[m] = sum_k G(m,k) f_X(m,k) N_k
// where beta = sum_X beta_X f_X. The -lambda_m - lambda_k part of G reduces to
// moments of N and of lambda*N (as the forward death term); the P part is a
// row gather: row m meets each partner k once as the smaller member
// ("upper", lo = m + Ld[k-m]) and once as the larger ("lower",
// lo = k + Ld[m-k]). P uses the reference's weight numerator fl(x_j + x_k) -
// x_lo (integer pipe) times (lambda_{lo+1} - lambda_lo)/(x_{lo+1} - x_lo).
// One CTA owns each row tile and reduces it in a fixed order -> deterministic.
//
// Breakage. rhs_i = -S_i N_i + sum_j S_j N_j sum_q bw_q eta_i(x_j t_q) over
// the guarded parents. With Q_j = -lambda_j + sum_q bw_q P_jq:
//   dL/dN_j = S_j Q_j, dL/dS0 = sum_j (S_j/S0) N_j Q_j, dL/dv_ref, dL/dalpha
// (PowerLaw: dS/dalpha = S ln(x/v_ref)), dL/dv_min = 0 (threshold step).
// =============================================================================
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "pbe_internal.cuh"
#include "vjp_tile.cuh"

namespace pbe_gb300 {
namespace {

constexpr int VW = kVW;                 // rows per task

// dL/dN needs, per kernel type K, up to two row sums (see vjp_main_kernel):
//   K=0: R0 = sum P N_k                       f = 1
//   K=1: R0 = sum P N_k, R1 = sum P h_k       f N_k = x_m N_k + h_k
//   K=2: R0 = sum P h_k                       f N_k = x_m h_k
//   K=3: R0 = sum P N_k Bf                    Brownian factor per lag
//   K=4: R1 = sum_upper P N_k Sf + sum_lower P N_k Sl (shear f = x_min Sf;
//        on a geometric grid x_min = x_k = x_m x_0/x_d for a lower partner, so
//        f = x_m Sl with Sl = Sf x_0/x_d and both visits sum into R1, times x_m)
//   K=5: R0, R1 as K=3 and K=4
// The generic (non-geometric) path accumulates sum P N_k f directly: R0 for
// K=0..3 (f = f_0 or Bf), R1 for the shear part.

// -------------------------------------------------------------------------
// prep: per-bin values, lag factors (no beta, no diagonal 1/2), moments of N
// and lambda*N, geometric deviation. Moment slots per block (stride 16):
// 0..4 sum N{1/a, 1, a, a^2, x}, 5..9 the same of lambda*N, 10 max dev.
// Modes: kVjpFull everything; kVjpTables the grid-only part (cube roots, lag
// tables, bracket offsets, deviation) for callers that keep the workspace for
// one set of pivots (the RK4 tape); kVjpStage the N- and lambda-dependent
// part (x N, D, moments) on such a workspace, with kVjpFull's arithmetic.
// -------------------------------------------------------------------------
enum { kVjpFull = 0, kVjpTables = 1, kVjpStage = 2 };

template <int MODE>
__global__ void __launch_bounds__(kPrepThreads)
vjp_prep_kernel(const double* __restrict__ N, const double* __restrict__ x,
                const double* __restrict__ lam, int n, VjpWs ws)
{
    __shared__ double sh[kPrepThreads / 32];
    __shared__ double ax0_s;
    __shared__ GeoFit fit_s;
    const int i = blockIdx.x * kPrepThreads + threadIdx.x;
    if constexpr (MODE != kVjpStage) {
        if (threadIdx.x == 0) {
            ax0_s = cbrt(x[0]);
            fit_s = geo_fit(x[0], x[n - 1], n);
        }
        __syncthreads();
    }
    double m[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) m[q] = 0.0;
    double dev = 0.0;
    if (i < n) {
        const double xi = x[i];
        double ai, iai;
        if constexpr (MODE == kVjpStage) {
            ai = ws.a[i];
            iai = ws.ia[i];
        } else {
            ai = cbrt(xi);
            iai = 1.0 / ai;
            ws.a[i] = ai;
            ws.ia[i] = iai;
            const double x0 = x[0];
            const double rho = ai / ax0_s;
            ws.Bf[i] = rho + 1.0 / rho + 2.0;
            const double s = 1.0 + rho;
            ws.Sf[i] = (s * s) * s;
            ws.Sl[i] = (s * s) * s * (x0 / xi);
            const double v = x0 + xi;
            ws.Ld[i] = (dbits(v) >= dbits(x[n - 1])) ? kLagClipAll : bracket_from(x, n, v, i);
            // launch order of the lane tasks: entry i < full is a full chunk
            // (chunk by chunk), entry full + rank(b) row block b's last chunk
            const int C = vjp_lane_chunk(n);
            const int full = vjp_lane_full_tasks(n, C);
            if (i < full) {
                int r = i, c = 0;
                for (;;) {
                    const int cnt = vjp_lane_chunk_blocks(n, c + 1, C);
                    if (r < cnt) break;
                    r -= cnt;
                    ++c;
                }
                ws.ltask[2 * i] = r;
                ws.ltask[2 * i + 1] = c;
            }
            if (i < vjp_lane_chunk_blocks(n, 0, C)) {
                const int dmax = n - 1 - kLaneBins * i;
                const int k = full + vjp_lane_last_rank(n, i, C);
                ws.ltask[2 * k] = i;
                ws.ltask[2 * k + 1] = (dmax + C - 1) / C - 1;
            }
            if (n >= 2) {
                dev = geo_dev(fit_s, xi, i);
                if (!(dev == dev)) dev = 1.0;
            }
        }
        if constexpr (MODE != kVjpTables) {
            const double Ni = N[i], li = lam[i];
            ws.h[i] = xi * Ni;
            ws.D[i] = (i < n - 1) ? (lam[i + 1] - li) / (x[i + 1] - xi) : 0.0;
            const double w[5] = {iai, 1.0, ai, ai * ai, xi};
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                m[q] = w[q] * Ni;
                m[5 + q] = w[q] * (li * Ni);
            }
        }
    }
    if constexpr (MODE != kVjpTables) {
#pragma unroll
        for (int q = 0; q < 10; ++q) {
            const double s = block_sum(m[q], sh);
            if (threadIdx.x == 0) ws.mom_part[blockIdx.x * 16 + q] = s;
        }
    }
    if constexpr (MODE != kVjpStage) {
        dev = warp_max(dev);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dev;
        __syncthreads();
        if (threadIdx.x == 0) {
            double mx = 0.0;
            for (int w = 0; w < kPrepThreads / 32; ++w) mx = fmax(mx, sh[w]);
            ws.mom_part[blockIdx.x * 16 + 10] = mx;
        }
    }
}

// One block: the reductions over the prep blocks' partials, one per warp and
// round (lanes stride over the blocks, fixed butterflies): the ten moments
// (kVjpFull, kVjpStage) and the geometric flag (kVjpFull, kVjpTables); resets
// the task counters (kVjpFull, kVjpStage).
template <int MODE>
__global__ void __launch_bounds__(256)
vjp_fin_kernel(const double* __restrict__ x, int n, VjpWs ws)
{
    __shared__ double mx_s;
    const int nb = (n + kPrepThreads - 1) / kPrepThreads;
    const int wq = threadIdx.x >> 5, lq = threadIdx.x & 31;
    for (int r = wq; r < 11; r += 8) {
        double t = 0.0;
        if (r < 10) {
            if (MODE == kVjpTables) continue;
            for (int b = lq; b < nb; b += 32) t += ws.mom_part[b * 16 + r];
            t = warp_sum(t);
            if (lq == 0) ws.mom[r] = t;
        } else {
            if (MODE == kVjpStage) continue;
            for (int b = lq; b < nb; b += 32) t = fmax(t, ws.mom_part[b * 16 + 10]);
            t = warp_max(t);
            if (lq == 0) mx_s = t;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (MODE != kVjpStage) {
            const bool ratio_ok = n >= 2 && x[1] <= 64.0 * x[0];
            ws.mom[10] = (n >= 2 && mx_s <= kGeoTol && ratio_ok) ? 1.0 : 0.0;
        }
        if (MODE != kVjpTables) {
            ws.counter[0] = 0;
            ws.counter[1] = 0;
        }
    }
}

// Pair sums: task = (row tile, partner chunk); the whole CTA is one group.
// Each task stores its rows' two sums per chunk; vjp_rows_kernel adds the
// chunks in order and finishes the rows.
// lane_on: the lane-block kernel takes geometric grids (this one returns).
template <int K>
__global__ void __launch_bounds__(kMainThreads, 2)
vjp_main_kernel(const double* __restrict__ N, const double* __restrict__ x,
                const double* __restrict__ lam, VjpWs ws, int n, int ntile, int nch, int lane_on)
{
    extern __shared__ double red[];               // [kVRows][kMainThreads]
    __shared__ VjpShared sm;
    __shared__ int s_task;

    if (lane_on && ws.mom[10] != 0.0) return;
    const int tid = threadIdx.x;
    VjpCellView v;
    v.x = x; v.N = N; v.h = ws.h; v.lam = lam; v.D = ws.D; v.a = ws.a; v.ia = ws.ia;
    v.Bf = ws.Bf; v.Sf = ws.Sf; v.Sl = ws.Sl; v.Ld = ws.Ld; v.lag0_scale = 1.0;
    v.n = n;
    v.geo = ws.mom[10] != 0.0;
    const TileGroup G{0, tid, kMainThreads};
    const int span = (n + nch - 1) / nch;

    for (;;) {
        if (tid == 0) s_task = atomicAdd(ws.counter, 1);
        __syncthreads();
        const int task = s_task;
        __syncthreads();
        if (task >= ntile * nch) break;
        const int tile = task / nch, chunk = task - tile * nch;
        const int r0 = min(n, chunk * span), r1 = min(n, r0 + span);
        vjp_tile_accumulate<K>(v, tile * VW, r0, r1, red, sm, G);
        if (tid < kVRows) ws.vpart[(static_cast<size_t>(tile) * nch + chunk) * kVRows + tid] = sm.fin[0][tid];
        __syncthreads();
    }
}

// Rows: one warp per row tile. Sums the tile's chunks in order, adds each
// row's dL/dN_m and stores the tile's parameter partials (fixed order).
template <int K>
__global__ void __launch_bounds__(256)
vjp_rows_kernel(const double* __restrict__ N, const double* __restrict__ x,
                const double* __restrict__ lam, double* __restrict__ gN, VjpWs ws, int n,
                int ntile, int nch, double b0, double bbr, double bsh, int lane_on)
{
    __shared__ double fin[8][kVRows];
    if (lane_on && ws.mom[10] != 0.0) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * 8 + w;
    if (tile >= ntile) return;                    // whole warp
    for (int r = lane; r < kVRows; r += 32) {
        double s = 0.0;
        for (int c = 0; c < nch; ++c) s += ws.vpart[(static_cast<size_t>(tile) * nch + c) * kVRows + r];
        fin[w][r] = s;
    }
    __syncwarp();
    VjpCellView v;
    v.x = x; v.N = N; v.h = ws.h; v.lam = lam; v.D = ws.D; v.a = ws.a; v.ia = ws.ia;
    v.Bf = ws.Bf; v.Sf = ws.Sf; v.Sl = ws.Sl; v.Ld = ws.Ld; v.lag0_scale = 1.0;
    v.n = n;
    v.geo = ws.mom[10] != 0.0;
    const int I = tile * VW;
    double gB = 0.0, gS = 0.0;
    if (lane < VW && I + lane < n) {
        double g;
        vjp_tile_row<K>(v, I + lane, lane, fin[w], ws.mom, ws.mom + 5, b0, bbr, bsh, g, gB, gS);
        gN[I + lane] += g;
    }
    double s0 = 0.0, s1 = 0.0;
    for (int t = 0; t < VW; ++t) {
        s0 += __shfl_sync(0xffffffffu, gB, t);
        s1 += __shfl_sync(0xffffffffu, gS, t);
    }
    if (lane == 0) {
        // slots: 0 beta0, 1 beta_br, 2 beta_sh
        ws.gpart[tile * 4 + 0] = (K <= 2) ? s0 : 0.0;
        ws.gpart[tile * 4 + 1] = (K == 3 || K == 5) ? s0 : 0.0;
        ws.gpart[tile * 4 + 2] = (K == 4 || K == 5) ? s1 : 0.0;
    }
}

// gp[0..nslots) += fixed-order sums of the per-tile partials
// One block: parameter slot q (< nslots <= 4) summed by warp q over the
// tasks' partials in a fixed order. nlane > 0: on a geometric grid the lane
// rows kernel wrote nlane partials instead of ntile.
__global__ void __launch_bounds__(128) vjp_gfin_kernel(int ntile, VjpWs ws, double* gp, int nslots,
                                                       int nlane)
{
    const int q = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (q >= nslots) return;
    if (nlane > 0 && ws.mom[10] != 0.0) ntile = nlane;
    double s = 0.0;
    for (int b = l; b < ntile; b += 32) s += ws.gpart[b * 4 + q];
    s = warp_sum(s);
    if (l == 0) gp[q] += s;
}

// -------------------------------------------------------------------------
// Lane blocks (geometric grids). Lane l of a warp owns row j = 32 b + l and
// walks the lags d of its share: the pair (j, k = j + d) lands at
// lo = j + Ld[d], P = lambda_lo + (fl(x_j + x_k) - x_lo) D_lo (lambda_{n-1} when
// clipped). The row of the smaller member sums in registers (U0, U1: the
// tile path's sums of the upper visits); the row of the larger member,
// k = j + d, is the row lane l + 1 held one lag earlier, so its sum W (the
// whole lower-visit term, parameters included) moves one lane down per lag;
// lane 0's finished W leaves the warp each lag into a shared window, and
// every lane's W at the end of the share. Brownian + shear: 7 FP64
// instructions per pair (P; P Bf, P Sf; two sums of the smaller member; two
// FMAs into W) against 8 for the two visits of the tile path.
// Tasks (row block, lag chunk) run largest first from the prep's launch-order
// table. Determinism: the windows of the CTA's warps are added in warp order;
// the rows kernel adds the tasks' sums in a fixed order.
// -------------------------------------------------------------------------
#ifndef PBE_VJP_LANE_CTAS
#define PBE_VJP_LANE_CTAS 3
#endif
constexpr int kVLaneCtas = PBE_VJP_LANE_CTAS;
constexpr int kLaneWarps = kMainThreads / 32;   // warps sharing a task's lags
#ifdef PBE_VJP_UNROLL
constexpr int kVjpUnroll = PBE_VJP_UNROLL;
#endif
constexpr int kVLaneMaxChunks = 64;        // vjp_lane_chunks(n, C) bound

template <int K>
__global__ void __launch_bounds__(kMainThreads, kVLaneCtas)
vjp_lane_kernel(const double* __restrict__ N, const double* __restrict__ x,
                const double* __restrict__ lam, VjpWs ws, int n, int ntasks, int C,
                double b0, double bbr, double bsh)
{
    extern __shared__ double esm[];               // [kLaneWarps][per_max + 32] W windows
    __shared__ double red[kLaneWarps][2][kLaneBins];
    __shared__ int s_task;

    if (ws.mom[10] == 0.0) return;                // not geometric: the tile kernel runs
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const double* __restrict__ h = ws.h;
    const double* __restrict__ D = ws.D;
    const int* __restrict__ Ld = ws.Ld;
    const double lamlast = lam[n - 1];
    const int ew = (C + kLaneWarps - 1) / kLaneWarps + 32;
    double* eb = esm + w * ew;

    for (;;) {
        if (tid == 0) s_task = atomicAdd(ws.counter + 1, 1);
        __syncthreads();
        const int task = s_task;
        __syncthreads();
        if (task >= ntasks) break;
        // largest first (the prep's launch order); the sums are stored under the
        // chunk-major index sum_{c' < c} blocks(c') + b that the rows kernel reads
        const int b = __ldg(ws.ltask + 2 * task), c = __ldg(ws.ltask + 2 * task + 1);
        int tix = b;
        for (int q = 0; q < c; ++q) tix += vjp_lane_chunk_blocks(n, q, C);
        const int J = kLaneBins * b;
        const int dA = 1 + c * C;
        const int dB = min(dA + C, n - J);        // lags [dA, dB), dB - 1 <= n - 1 - J
        const int len = dB - dA;
        const int per = (len + kLaneWarps - 1) / kLaneWarps;
        const int dw0 = dA + w * per;
        const int dw1 = min(dB, dw0 + per);

        const int j = J + lane;
        const bool jv = j < n;
        const double xj = jv ? __ldg(x + j) : 0.0;
        const double Nj = jv ? __ldg(N + j) : 0.0;
        const double hj = jv ? h[j] : 0.0;
        // lane constants of the lower-visit term
        double cN = 0.0, cH = 0.0;
        if constexpr (K == 0) cN = b0 * Nj;
        if constexpr (K == 1) { cN = b0 * Nj; cH = b0 * hj; }
        if constexpr (K == 2) cH = b0 * hj;
        if constexpr (K == 3) cN = bbr * Nj;
        if constexpr (K == 4) cH = bsh * hj;
        if constexpr (K == 5) { cN = bbr * Nj; cH = bsh * hj; }
        const int jtop = n - 1 - j;               // lo >= n - 1 <=> Ld[d] >= jtop
        const EwOperandB pb = ew_operand_b(jv ? xj : 1.0);   // the row's pivot, decoded once

        double U0 = 0.0, U1 = 0.0, W = 0.0;
#ifdef PBE_VJP_UNROLL
#pragma unroll kVjpUnroll
#endif
        for (int d = dw0; d < dw1; ++d) {
            // lane 0's row (j + d - 1) is complete: out; every row moves one lane down
            const double Wd = __shfl_down_sync(0xffffffffu, W, 1);
            if (lane == 0) eb[d - dw0] = W;
            W = (lane == 31) ? 0.0 : Wd;
            const int L = __ldg(Ld + d);
            double Bf = 0.0, Sf = 0.0;
            if constexpr (K == 3 || K == 5) Bf = __ldg(ws.Bf + d);
            if constexpr (K == 4 || K == 5) Sf = __ldg(ws.Sf + d);
            const int k = j + d;
            if (k < n) {
                const double xk = __ldg(x + k);
                double P = lamlast;
                if (L < jtop) {
                    const int lo = j + L;
                    P = fma(sum_minus_scaled_dec(ew_operand_a(xk), pb, ew_operand_c(__ldg(x + lo), 0)),
                            D[lo], lam[lo]);
                }
                if constexpr (K == 0) {
                    U0 = fma(P, __ldg(N + k), U0);
                    W = fma(P, cN, W);
                } else if constexpr (K == 1) {
                    U0 = fma(P, __ldg(N + k), U0);
                    U1 = fma(P, h[k], U1);
                    W = fma(P, fma(cN, xk, cH), W);
                } else if constexpr (K == 2) {
                    U0 = fma(P, h[k], U0);
                    W = fma(P * xk, cH, W);
                } else {
                    const double Nk = __ldg(N + k);
                    if constexpr (K == 3 || K == 5) {
                        const double u0 = P * Bf;
                        U0 = fma(u0, Nk, U0);
                        W = fma(u0, cN, W);
                    }
                    if constexpr (K == 4 || K == 5) {
                        const double u1 = P * Sf;
                        U1 = fma(u1, Nk, U1);
                        W = fma(u1, cH, W);
                    }
                }
            }
        }
        if (dw1 > dw0) eb[dw1 - dw0 + lane] = W;  // rows j + dw1 - 1
        red[w][0][lane] = U0;
        red[w][1][lane] = U1;
        __syncthreads();
        if (w == 0) {
            double s0 = 0.0, s1 = 0.0;
#pragma unroll
            for (int q = 0; q < kLaneWarps; ++q) {
                s0 += red[q][0][lane];
                s1 += red[q][1][lane];
            }
            ws.lup[static_cast<size_t>(tix) * 2 * kLaneBins + lane] = s0;
            ws.lup[static_cast<size_t>(tix) * 2 * kLaneBins + kLaneBins + lane] = s1;
        }
        // the task's window: entry i is row J + dA - 1 + i, i < len + 32; warp q's
        // window starts at i = q per and holds its share's length + 32 entries
        double* seg = ws.llo + static_cast<size_t>(tix) * (C + 32);
        for (int i = tid; i < len + 32; i += kMainThreads) {
            double sum = 0.0;
            for (int q = 0; q < kLaneWarps; ++q) {
                const int q0 = q * per, q1 = min(len, q0 + per);
                if (q1 <= q0) break;
                const int o = i - q0;
                if (o >= 0 && o < q1 - q0 + 32) sum += esm[q * ew + o];
            }
            seg[i] = sum;
        }
        __syncthreads();
    }
}

// Rows of the lane path: one CTA per row block b (rows 32 b + lane). Warp g
// adds the larger-member sums of the row blocks b' = g, g + 32, ... <= b (the
// chunk holding lag d = m - 32 b' and, for the first 32 lags of a chunk, the
// tail of the chunk before); warp 0 adds the 32 in order, the block's own
// smaller-member sums chunk by chunk, the diagonal pair, the death moments,
// and stores dL/dN_m and the block's parameter partials.
#ifndef PBE_VROWS_WARPS
#define PBE_VROWS_WARPS 32
#endif
constexpr int kVRowsWarps = PBE_VROWS_WARPS;

template <int K>
__global__ void __launch_bounds__(kVRowsWarps * 32)
vjp_lane_rows_kernel(const double* __restrict__ N, const double* __restrict__ x,
                     const double* __restrict__ lam, double* __restrict__ gN, VjpWs ws, int n,
                     int C, double b0, double bbr, double bsh)
{
    __shared__ double lw[kVRowsWarps][kLaneBins];
    __shared__ int base[kVLaneMaxChunks + 1];
    if (ws.mom[10] == 0.0) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = gridDim.x - 1 - blockIdx.x;      // top row blocks (the most lower blocks) first
    const int m = kLaneBins * b + lane;
    const int nchunks = vjp_lane_chunks(n, C);
    if (threadIdx.x == 0) {
        int sacc = 0;
        for (int c = 0; c < nchunks; ++c) {
            base[c] = sacc;
            sacc += vjp_lane_chunk_blocks(n, c, C);
        }
    }
    __syncthreads();
    const size_t S = static_cast<size_t>(C) + 32;
    double acc = 0.0;
    if (m < n) {
        // the loads of several row blocks in flight: addresses do not depend on acc
        const float invC = 1.0f / static_cast<float>(C);
#pragma unroll 4
        for (int bp = w; bp <= b; bp += kVRowsWarps) {
            const int d = m - kLaneBins * bp;
            // c1 = d / C: the float quotient, corrected by one either way
            int c1 = __float2int_rz(static_cast<float>(d) * invC);
            c1 -= (c1 * C > d) ? 1 : 0;
            c1 += ((c1 + 1) * C <= d) ? 1 : 0;
            const int idx = d - c1 * C;
            double v = 0.0;
            if (d >= 1) {
                if (c1 >= 1 && idx < 32) v = __ldcg(ws.llo + (base[c1 - 1] + bp) * S + C + idx);
                // chunk c1 exists for block bp when its first lag 1 + c1 C <= n - 1 - 32 bp
                if (1 + c1 * C <= n - 1 - kLaneBins * bp) v += __ldcg(ws.llo + (base[c1] + bp) * S + idx);
            }
            acc += v;
        }
    }
    lw[w][lane] = acc;
    __syncthreads();
    if (w != 0) return;

    double gB = 0.0, gS = 0.0;
    if (m < n) {
        double Wm = 0.0;
#pragma unroll
        for (int q = 0; q < kVRowsWarps; ++q) Wm += lw[q][lane];
        const int dmax = n - 1 - kLaneBins * b;
        const int nchb = dmax >= 1 ? (dmax + C - 1) / C : 0;
        double U0 = 0.0, U1 = 0.0;
        for (int c = 0; c < nchb; ++c) {
            const double* up = ws.lup + static_cast<size_t>(base[c] + b) * 2 * kLaneBins;
            U0 += __ldcg(up + lane);
            U1 += __ldcg(up + kLaneBins + lane);
        }
        // diagonal pair (m, m), counted once
        const double xm = x[m], Nm = N[m], hm = ws.h[m], lm = lam[m];
        const int L0 = ws.Ld[0];
        double P = lam[n - 1];
        if (L0 < n - 1 - m) {
            const int lo = m + L0;
            P = fma(sum_minus_scaled(xm, xm, x[lo], 0), ws.D[lo], lam[lo]);
        }
        double d0 = 0.0, d1 = 0.0;
        if constexpr (K == 0) d0 = P * Nm;
        if constexpr (K == 1) { d0 = P * Nm; d1 = P * hm; }
        if constexpr (K == 2) d0 = P * hm;
        if constexpr (K == 3 || K == 5) d0 = (P * Nm) * ws.Bf[0];
        if constexpr (K == 4 || K == 5) d1 = (P * Nm) * ws.Sf[0];
        U0 += d0;
        U1 += d1;
        // Tv: the smaller-member sums (diagonal included) weighted as the kernel
        // factor f(m, k) N_k; Td: the diagonal's share
        double Tv0 = U0, Td0 = d0, Tv1 = 0.0, Td1 = 0.0;
        if constexpr (K == 1) { Tv0 = fma(xm, U0, U1); Td0 = fma(xm, d0, d1); }
        if constexpr (K == 2) { Tv0 = xm * U0; Td0 = xm * d0; }
        if constexpr (K == 4 || K == 5) { Tv1 = xm * U1; Td1 = xm * d1; }
        const double am = ws.a[m], iam = ws.ia[m];
        const double* M = ws.mom;
        const double* Lm = ws.mom + 5;
        double g = Wm;
        if constexpr (K != 4) {
            const double dth0 = fma(lm, moment_factor<K, 0>(xm, am, iam, M), moment_factor<K, 0>(xm, am, iam, Lm));
            const double coef = (K <= 2) ? b0 : bbr;
            g = fma(coef, Tv0 - dth0, g);
            gB = Nm * Tv0 - 0.5 * Nm * (Td0 + dth0);
        }
        if constexpr (K == 4 || K == 5) {
            const double dth1 = fma(lm, moment_factor<K, 1>(xm, am, iam, M), moment_factor<K, 1>(xm, am, iam, Lm));
            g = fma(bsh, Tv1 - dth1, g);
            gS = Nm * Tv1 - 0.5 * Nm * (Td1 + dth1);
        }
        gN[m] += g;
    }
    const double s0 = warp_sum(gB);
    const double s1 = warp_sum(gS);
    if (lane == 0) {
        // slots: 0 beta0, 1 beta_br, 2 beta_sh
        ws.gpart[b * 4 + 0] = (K <= 2) ? s0 : 0.0;
        ws.gpart[b * 4 + 1] = (K == 3 || K == 5) ? s0 : 0.0;
        ws.gpart[b * 4 + 2] = (K == 4 || K == 5) ? s1 : 0.0;
    }
}

// -------------------------------------------------------------------------
// breakage VJP: nqp lanes per parent j (nqp = n_quad rounded up to a power of
// two, <= 32), each lane the fragments q = l % nqp, + nqp, ... (their bracket
// searches run side by side), summed over the lanes by a fixed butterfly;
// block partials of the parameter sums.
// -------------------------------------------------------------------------
template <int F>
__global__ void __launch_bounds__(256)
brk_vjp_kernel(const double* __restrict__ N, const double* __restrict__ x,
               const double* __restrict__ t_q, const double* __restrict__ bw_q,
               const double* __restrict__ lam, double* __restrict__ gN, double* part, int n,
               int nq, int nqp, double S0, double v_ref, double alpha, double v_min,
               const double* __restrict__ Ssel, const int* __restrict__ lo_tab)
{
    __shared__ double sh[8];
    const int l = threadIdx.x % nqp;
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) / nqp;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    double S = 0.0, Nj = 0.0, xj = 1.0;
    bool on = false;
    double acc = 0.0;
    const float lx0 = log2_approx(__ldg(x));
    const float span = log2_approx(__ldg(x + n - 1)) - lx0;
    const float inv_span = (n > 1 && span > 0.0f) ? static_cast<float>(n - 1) / span : 0.0f;
    if (j < n) {
        xj = x[j];
        Nj = N[j];
        S = Ssel ? Ssel[j] : selection<F>(xj, S0, v_ref, alpha, v_min);
        on = (S != 0.0) && (Nj > kBreakageNMin);
        if (on) {
            for (int q = l; q < nq; q += nqp) {
                const double v = xj * t_q[q];
                const int lo = lo_tab ? lo_tab[static_cast<size_t>(q) * n + j]
                                      : frag_bracket_guess(x, n, v, lx0, inv_span);
                double P;
                if (lo < 0) P = lam[0];
                else if (lo >= n - 1) P = lam[n - 1];
                else {
                    const double xl = x[lo], xh = x[lo + 1];
                    const double eta = (v - xl) / (xh - xl);
                    P = fma(1.0 - eta, lam[lo], eta * lam[lo + 1]);
                }
                acc = fma(bw_q[q], P, acc);
            }
        }
    }
    for (int o = nqp >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (on && l == 0) {
        const double Q = acc - lam[j];
        gN[j] += S * Q;
        const double NQ = Nj * Q;
        p0 = (S / S0) * NQ;
        if constexpr (F == 1) p1 = -(S / v_ref) * NQ;
        if constexpr (F == 2) {
            p1 = -(alpha * S / v_ref) * NQ;
            p2 = S * log(xj / v_ref) * NQ;
        }
    }
    const double s0 = block_sum(p0, sh);
    const double s1 = block_sum(p1, sh);
    const double s2 = block_sum(p2, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 4 + 0] = s0;
        part[blockIdx.x * 4 + 1] = s1;
        part[blockIdx.x * 4 + 2] = s2;
        part[blockIdx.x * 4 + 3] = 0.0;
    }
}

// Partner chunks per row tile: the row tiles cost the same, so with ntile
// tasks on 2 num_sms CTA slots the last wave can run half empty; pick the
// chunk count (<= kVjpMaxChunks, chunks of >= 512 partners) whose waves come
// closest to whole numbers, the smaller count on near ties.
int vjp_chunks(int ntile, int num_sms, int n)
{
    const double slots = 2.0 * num_sms;
    int best = 1;
    double best_eff = 0.0;
    for (int c = 1; c <= kVjpMaxChunks; ++c) {
        if (c > 1 && n / c < 512) break;
        const double w = ntile * c / slots;
        const double eff = w / std::ceil(w);
        if (eff > best_eff + 0.02) { best_eff = eff; best = c; }
    }
    return best;
}

// Aggregation VJP pair sums on geometric grids: lane blocks (default) or the
// row tiles of every grid. PBE_GB300_VJP_PATH=tile selects the tiles.
int vjp_lane_mode()
{
    static const int mode = []() {
        const char* e = std::getenv("PBE_GB300_VJP_PATH");
        return (e && std::strcmp(e, "tile") == 0) ? 0 : 1;
    }();
    return mode;
}

template <int K>
cudaError_t agg_vjp_k(const AggVjpArgs& a, const VjpWs& ws, int num_sms, cudaStream_t s, int kind)
{
    const int n = a.n;
    const int nb = (n + kPrepThreads - 1) / kPrepThreads;
    const int ntile = (n + VW - 1) / VW;
    const int nch = vjp_chunks(ntile, num_sms, n);
    const int ntasks = ntile * nch;
    const int grid = ntasks < 2 * num_sms ? ntasks : 2 * num_sms;
    const size_t smem = sizeof(double) * kVRows * kMainThreads;
    cudaError_t e = cudaFuncSetAttribute(vjp_main_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const int C = vjp_lane_chunk(n);
    const long long ltasks = vjp_lane_tasks(n, C);
    const int lane_on = (vjp_lane_mode() && ltasks > 0 && vjp_lane_chunks(n, C) <= kVLaneMaxChunks) ? 1 : 0;
    if (kind == kVjpTables) {
        vjp_prep_kernel<kVjpTables><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, a.lam, n, ws);
        vjp_fin_kernel<kVjpTables><<<1, 256, 0, s>>>(a.x, n, ws);
        return cudaGetLastError();
    }
    if (kind == kVjpStage) {
        vjp_prep_kernel<kVjpStage><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, a.lam, n, ws);
        vjp_fin_kernel<kVjpStage><<<1, 256, 0, s>>>(a.x, n, ws);
    } else {
        vjp_prep_kernel<kVjpFull><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, a.lam, n, ws);
        vjp_fin_kernel<kVjpFull><<<1, 256, 0, s>>>(a.x, n, ws);
    }
    const int nrb = (n + kLaneBins - 1) / kLaneBins;
    if (lane_on) {
        const size_t lsmem = sizeof(double) * kLaneWarps * ((C + kLaneWarps - 1) / kLaneWarps + 32);
        const int lgrid = static_cast<int>(ltasks < kVLaneCtas * num_sms ? ltasks : kVLaneCtas * num_sms);
        vjp_lane_kernel<K><<<lgrid, kMainThreads, lsmem, s>>>(a.N, a.x, a.lam, ws, n,
                                                              static_cast<int>(ltasks), C,
                                                              a.beta0, a.beta_br, a.beta_sh);
    }
    vjp_main_kernel<K><<<grid, kMainThreads, smem, s>>>(a.N, a.x, a.lam, ws, n, ntile, nch, lane_on);
    vjp_rows_kernel<K><<<(ntile + 7) / 8, 256, 0, s>>>(a.N, a.x, a.lam, a.gN, ws, n, ntile, nch,
                                                       a.beta0, a.beta_br, a.beta_sh, lane_on);
    if (lane_on)
        vjp_lane_rows_kernel<K><<<nrb, kVRowsWarps * 32, 0, s>>>(a.N, a.x, a.lam, a.gN, ws, n, C, a.beta0,
                                                    a.beta_br, a.beta_sh);
    vjp_gfin_kernel<<<1, 128, 0, s>>>(ntile, ws, a.gp, 3, lane_on ? nrb : 0);
    return cudaGetLastError();
}

template <int F>
cudaError_t brk_vjp_f(const BrkVjpArgs& a, const VjpWs& ws, cudaStream_t s, const double* Ssel,
                      const int* lo_tab)
{
    int nqp = 1;
    while (nqp < a.n_quad && nqp < 32) nqp <<= 1;
    const int nb = static_cast<int>((static_cast<long long>(a.n) * nqp + 255) / 256);
    brk_vjp_kernel<F><<<nb, 256, 0, s>>>(a.N, a.x, a.t_q, a.bw_q, a.lam, a.gN, ws.gpart, a.n,
                                         a.n_quad, nqp, a.S0, a.v_ref, a.alpha, a.v_min, Ssel,
                                         lo_tab);
    vjp_gfin_kernel<<<1, 128, 0, s>>>(nb, ws, a.gp, 4, 0);
    return cudaGetLastError();
}

} // namespace

namespace {
cudaError_t agg_vjp_dispatch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s, int kind)
{
    VjpWs ws;
    vjp_ws_layout(a.n, static_cast<char*>(ws_base), &ws);
    switch (a.kernel) {
    case 0: return agg_vjp_k<0>(a, ws, num_sms, s, kind);
    case 1: return agg_vjp_k<1>(a, ws, num_sms, s, kind);
    case 2: return agg_vjp_k<2>(a, ws, num_sms, s, kind);
    case 3: return agg_vjp_k<3>(a, ws, num_sms, s, kind);
    case 4: return agg_vjp_k<4>(a, ws, num_sms, s, kind);
    case 5: return agg_vjp_k<5>(a, ws, num_sms, s, kind);
    default: return cudaErrorInvalidValue;
    }
}
} // namespace

cudaError_t agg_vjp_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s)
{
    return agg_vjp_dispatch(a, ws_base, num_sms, s, kVjpFull);
}
cudaError_t agg_vjp_tables_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s)
{
    return agg_vjp_dispatch(a, ws_base, num_sms, s, kVjpTables);
}
cudaError_t agg_vjp_stage_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s)
{
    return agg_vjp_dispatch(a, ws_base, num_sms, s, kVjpStage);
}

cudaError_t brk_vjp_launch(const BrkVjpArgs& a, void* ws_base, cudaStream_t s, const double* Ssel,
                           const int* lo_tab)
{
    VjpWs ws;
    vjp_ws_layout(a.n, static_cast<char*>(ws_base), &ws);
    switch (a.selection) {
    case 0: return brk_vjp_f<0>(a, ws, s, Ssel, lo_tab);
    case 1: return brk_vjp_f<1>(a, ws, s, Ssel, lo_tab);
    case 2: return brk_vjp_f<2>(a, ws, s, Ssel, lo_tab);
    case 3: return brk_vjp_f<3>(a, ws, s, Ssel, lo_tab);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace pbe_gb300
