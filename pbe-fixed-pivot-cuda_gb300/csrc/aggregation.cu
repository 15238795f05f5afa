// =============================================================================
// aggregation.cu -- fixed-pivot aggregation RHS for GB300 (sm_103a), FP64.
//
// Reference semantics (acuoci/pbe-fixed-pivot-cuda src/aggregation_kernels.cuh:145-239):
// for every pair j <= k, rate = beta_jk N_j N_k (x1/2 if j == k); death -rate
// at j and at k (-2 rate on the diagonal); birth of v = x_j + x_k split onto
// the bracketing pivots lo, lo+1 with w = (v - x_lo)/(x_{lo+1} - x_lo); v >=
// x[n-1] goes wholly to bin n-1 (:191-192).
//
// Formulation used here (same sums, reorganised for an FP64-starved GPU):
//  * Death is separable: sum_k beta_ik N_k is a combination of five moments
//    M_p = sum_k x_k^p N_k (p = -1/3, 0, 1/3, 2/3, 1) for every kernel type,
//    so the death term costs O(n) instead of O(n^2).
//  * Birth is a gather over "slots": slot s collects the pairs whose bracket
//    is lo = s. Per slot two sums are kept, R_s = sum rate and
//    TH_s = sum rate * (v - x_s). Then bin i receives
//    (R_i - TH_i / dx_i) + TH_{i-1} / dx_{i-1}, which is the reference's
//    (1 - w) rate + w rate regrouped.
//  * Geometric grids (verified on the device, see agg_prep_kernel): the
//    bracket offset lo - j, the Brownian factor and the shear factor depend on
//    the lag d = k - j only. They come from per-lag tables, so a pair costs
//    1-3 FP64 operations plus two accumulations. The weight numerator
//    fl(x_j + x_k) - x_lo is formed from the actual pivots exactly as the
//    reference forms it, but on the integer pipe (exact_weight.cuh). For lags
//    whose pairs land on the larger member's own slot (lo = k, about half of
//    the pairs at n = 16384) N_k is a per-slot constant and is factored out.
//  * Generic grids: per-pair brackets by a monotone walk over k, beta from
//    per-bin cube roots.
//  * Pairs clipped at x[n-1] are summed by up to 32 extra tasks of the main
//    kernel (interleaved lags on a geometric grid, rows otherwise); in gather
//    mode the last of them and of the task owning bin n-1 adds their parts, in
//    order, to rhs[n-1].
//
// Kernels per call: prep (per-bin values, lag tables, moment partials,
// geometric check; its last block finishes moments, flag and counters) ->
// main (persistent CTAs pulling target tiles, or for small n their lag
// chunks, from an atomic counter, largest first). GATHER mode: each output
// bin is written once, from sums reduced in a fixed order -> bitwise
// reproducible. SCATTER mode: every task flushes its bins with FP64 atomicAdd.
// =============================================================================
#include <cstdlib>
#include <cstring>

#include "pbe_internal.cuh"
#include "agg_tile.cuh"
#include "agg_lane.cuh"

namespace pbe_gb300 {
namespace {

constexpr int W = kTileW;

// ---------------------------------------------------------------------------
// prep: one thread per bin i. Per-bin values, the lag tables for d = i,
// moment partials and the geometric-grid deviation.
//   Bd[d], Sd[d]: beta(x_j, x_{j+d}) = Bd + x_j Sd on a geometric grid, times
//   c_d (1/2 for d = 0), with rho = x_d^(1/3) / x_0^(1/3):
//     Constant/Sum/Product: Bd = c_d beta0 (the x dependence stays per pair)
//     Brownian: Bd = c_d beta_br (rho + 1/rho + 2)
//     Shear:    Sd = c_d beta_sh (1 + rho)^3
//   Ld[d]: bracket of x_0 + x_d (kLagClipAll when it reaches x[n-1]).
//
// FULL = false (stage calls of a caller that keeps the workspace, e.g. the RK4
// tape): every grid-only entry -- a, ia, inv_dx, the x copy, Bd, Sd, Ld, the
// geometric flag mom[5..6] and D0 in counter[1] -- is left as an earlier FULL
// call on the same pivots and coefficients wrote it; only the N-dependent
// values (h, the N copy, moments) and the tickets are rewritten, with the
// same arithmetic as a FULL call, so the results are bitwise the same.
// Either way the last block resets counter[2] (the prep's block tickets), so
// a following call on the same workspace needs no memset.
// ---------------------------------------------------------------------------
template <int K, bool FULL>
__global__ void __launch_bounds__(kPrepThreads)
agg_prep_kernel(const double* __restrict__ N, const double* __restrict__ x, int n, AggWs ws,
                double b0, double bbr, double bsh)
{
    __shared__ double sh[kPrepThreads / 32];
    __shared__ int d0_s;
    __shared__ double ax0_s;
    __shared__ GeoFit fit_s;
    const int i = blockIdx.x * kPrepThreads + threadIdx.x;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double dev = 0.0;
    int d0 = n;      // this thread's lag if its pairs land on their larger member (Ld == d)
    if (FULL && threadIdx.x == 0) {
        d0_s = n;
        ax0_s = cbrt(x[0]);
        fit_s = geo_fit(x[0], x[n - 1], n);
    }
    __syncthreads();
    if (i < n) {
        const double xi = x[i], Ni = N[i];
        const double hi = xi * Ni;
        double ai, iai;
        if constexpr (FULL) {
            ai = cbrt(xi);
            iai = 1.0 / ai;
        } else {
            ai = ws.a[i];
            iai = ws.ia[i];
        }
        ws.h[i] = hi;
        ws.Ncp[i] = Ni;          // 256-byte aligned copies: bulk-copy sources of the lane tasks
        m[0] = iai * Ni; m[1] = Ni; m[2] = ai * Ni; m[3] = (ai * ai) * Ni; m[4] = hi;
        if (i < agg_tiles(n)) { ws.tticket[i] = 0; ws.cticket[i] = 0; }
        if constexpr (FULL) {
            // launch order of the lane tasks: entry i < full is a full chunk
            // (chunk by chunk), entry full + rank(t) block t's last chunk
            const int C = lane_chunk_len(n);
            const int full = lane_full_tasks(n, C);
            if (i < full) {
                int r = i, c = 0;
                for (;;) {
                    const int cnt = lane_chunk_blocks(n, c + 1, C);
                    if (r < cnt) break;
                    r -= cnt;
                    ++c;
                }
                ws.ltask[2 * i] = r;
                ws.ltask[2 * i + 1] = c;
            }
            if (i < lane_blocks(n)) {
                const int k = full + lane_last_rank(n, i, C);
                ws.ltask[2 * k] = i;
                ws.ltask[2 * k + 1] = lane_block_chunks(n, i, C) - 1;
            }
            ws.xcp[i] = xi;
            ws.a[i] = ai;
            ws.ia[i] = iai;
            ws.inv_dx[i] = (i < n - 1) ? 1.0 / (x[i + 1] - xi) : 0.0;
            const double x0 = x[0];
            const double c = (i == 0) ? 0.5 : 1.0;
            double B = 0.0, S = 0.0;
            if constexpr (K <= 2) B = c * b0;
            if constexpr (K >= 3) {
                const double rho = ai / ax0_s;
                if constexpr (K == 3 || K == 5) B = c * bbr * (rho + 1.0 / rho + 2.0);
                if constexpr (K == 4 || K == 5) { const double s = 1.0 + rho; S = c * bsh * (s * s) * s; }
            }
            ws.Bd[i] = B;
            ws.Sd[i] = S;
            const double v = x0 + xi;       // x[i] <= v: its bracket is at or above i
            const int L = (dbits(v) >= dbits(x[n - 1])) ? kLagClipAll : bracket_from(x, n, v, i);
            ws.Ld[i] = L;
            if (L == i) d0 = i;
            if (n >= 2) {
                dev = geo_dev(fit_s, xi, i);
                if (!(dev == dev)) dev = 1.0;   // NaN -> not geometric
            }
        }
    }
    if (FULL) atomicMin(&d0_s, d0);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const double s = block_sum(m[q], sh);
        if (threadIdx.x == 0) ws.mom_part[blockIdx.x * 8 + q] = s;
    }
    if (FULL) {
        dev = warp_max(dev);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dev;
        __syncthreads();
    }
    __shared__ int last_s;
    if (threadIdx.x == 0) {
        if (FULL) {
            double mx = 0.0;
            for (int w = 0; w < kPrepThreads / 32; ++w) mx = fmax(mx, sh[w]);
            ws.mom_part[blockIdx.x * 8 + 5] = mx;
            ws.mom_part[blockIdx.x * 8 + 6] = static_cast<double>(d0_s);
        }
        __threadfence();                       // partials visible before the ticket
        last_s = (atomicAdd(ws.counter + 2, 1) == static_cast<int>(gridDim.x) - 1);
    }
    __syncthreads();
    if (!last_s) return;
    // The last block to finish reduces every block's partials (read through L2)
    // in a fixed order: moments, geometric flag, first lag with Ld[d] == d,
    // counters of the main kernel. No block waits for another.
    __threadfence();
    const int nb = gridDim.x;
    // seven reductions over the blocks' partials, spread over the warps: r < 5
    // one moment each, r = 5 the largest deviation, r = 6 the smallest D0
    // candidate (lanes stride over the blocks, fixed butterflies)
    const int wq = threadIdx.x >> 5, lq = threadIdx.x & 31;
    for (int r = wq; r < (FULL ? 7 : 5); r += kPrepThreads / 32) {
        if (r < 5) {
            double t = 0.0;
            for (int b = lq; b < nb; b += 32) t += __ldcg(ws.mom_part + b * 8 + r);
            t = warp_sum(t);
            if (lq == 0) ws.mom[r] = t;
        } else if (r == 5) {
            double m5 = 0.0;
            for (int b = lq; b < nb; b += 32) m5 = fmax(m5, __ldcg(ws.mom_part + b * 8 + 5));
            m5 = warp_max(m5);
            if (lq == 0) sh[0] = m5;
        } else {
            int dmin = n;
            for (int b = lq; b < nb; b += 32)
                dmin = min(dmin, static_cast<int>(__ldcg(ws.mom_part + b * 8 + 6)));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dmin = min(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
            if (lq == 0) d0_s = dmin;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (FULL) {
            const double mx = sh[0];
            // neighbour ratio <= 64 keeps fl(x_j + x_k) within kMaxExpGap binades of
            // its bracket pivot (precondition of sum_minus_scaled)
            const bool geo = n >= 2 && mx <= kGeoTol && x[1] <= 64.0 * x[0];
            ws.mom[5] = geo ? 1.0 : 0.0;
            ws.mom[6] = mx;
            ws.counter[1] = d0_s;   // lags d >= counter[1] have lo(j, j+d) = j + d
        }
        ws.counter[0] = 0;          // task counter of the main kernel
        ws.counter[2] = 0;          // this kernel's block tickets, ready for the next call
        ws.counter[3] = 0;          // contributors to bin n-1 done (clip tasks + top tile)
        ws.counter[4] = 0;          // lane-task staging error flag
    }
}

// Clipped pairs (x_j + x_k >= x[n-1], all deposited on bin n-1,
// src/aggregation_kernels.cuh:191-192), part c of nclip: the lags
// d = c + nclip (lane + T k) on a geometric grid (pairs j in [n-1-Ld, n-1-d];
// interleaving spreads the long lags near d = 0 over the parts), the rows
// j = c + nclip (lane + T k) otherwise.
template <int K>
__device__ double clip_part_sum(const AggCellView& v, int c, int nclip, const TileGroup& G)
{
    const int n = v.n;
    double acc = 0.0;
    if (v.geo) {
        for (int d = c + nclip * G.lane; d < n; d += nclip * G.T) {
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
        for (int j = c + nclip * G.lane; j < n; j += nclip * G.T) {
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

// Gather mode: the clip tasks and the task that owns bin n-1 each take a
// ticket after their contribution is stored; the last of the nclip + 1 adds
// the clip parts, in order, to rhs[n-1]. Called by one thread.
// (Bin n-1 is never a tile's first bin: tiles are aligned to the top.)
__device__ __forceinline__ void clip_contributor_done(double* rhs, int n, const AggWs& ws,
                                                      int nclip)
{
    __threadfence();
    if (atomicAdd(ws.counter + 3, 1) != nclip) return;
    __threadfence();
    double s = 0.0;
    for (int c = 0; c < nclip; ++c) s += __ldcg(ws.clip_part + c);
    rhs[n - 1] = __ldcg(rhs + (n - 1)) + s;
}

// Gather mode: tile `tile`'s first bin I receives the tile's own value and
// the carry of the tile below; each stores its part and takes a ticket, the
// second writes rhs[I] += own + carry (a sum of two: the same whichever is
// second). Called by one thread.
__device__ __forceinline__ void first_bin_done(double* rhs, int I, const AggWs& ws, int tile)
{
    __threadfence();
    if (atomicAdd(ws.tticket + tile, 1) != 1) return;
    __threadfence();
    rhs[I] = __ldcg(rhs + I) + (__ldcg(ws.tfirst + tile) + __ldcg(ws.tcarry + tile));
}

// ---------------------------------------------------------------------------
// main: persistent CTAs split into groups of T threads (agg_group_size); each
// group pulls tasks from the atomic counter on its own. Tiles are aligned to
// the top: tile t owns the W bins [I, I+W), I = n - W (t + 1) (the lowest tile
// may start below bin 0), and accumulates the slots s = I .. I+W-1 with the
// shared tile body (agg_tile.cuh). The w-part of slot I+W-1 belongs to bin
// I+W, the first bin of tile t-1: it is handed over as a carry, so each pair
// is evaluated once. Thread-private partial sums are reduced in a fixed
// order, so for a given T the gather result is bitwise reproducible.
// ---------------------------------------------------------------------------
template <int K, bool SCATTER>
__global__ void __launch_bounds__(kMainThreads, 2)
agg_main_kernel(const double* __restrict__ N, const double* __restrict__ x,
                double* __restrict__ rhs, AggWs ws, int n, int ntile,
                int ntasks, int nclip, double b0, double bbr, double bsh, int T, int Cg,
                int ntasks_lane)
{
    extern __shared__ double red[];               // [2 W][kMainThreads]
    __shared__ TileShared sm;
    __shared__ int s_task[kMaxGroups];
    __shared__ int s_last[kMaxGroups];

    const int tid = threadIdx.x;
    AggCellView v;
    v.x = x; v.Nk = N; v.Hk = ws.h; v.Nj = N; v.Hj = ws.h; v.Aj = N; v.AHj = ws.h;
    v.Fs = (K == 2) ? ws.h : N;
    v.a = ws.a; v.ia = ws.ia; v.inv_dx = ws.inv_dx;
    v.Bd = ws.Bd; v.Sd = ws.Sd; v.Ld = ws.Ld;
    v.n = n;
    v.D0 = ws.counter[1];
    v.geo = ws.mom[5] != 0.0;
    v.b0 = b0; v.bbr = bbr; v.bsh = bsh;
#pragma unroll
    for (int q = 0; q < 5; ++q) v.M[q] = ws.mom[q];

    // geometric grids run the lane-block kernel instead (launched just before)
    if (ntasks_lane > 0 && v.geo) return;

    // groups of T threads pull tasks on their own (no CTA-wide barrier in the loop)
    const int g = tid / T;
    const TileGroup G{g, tid - g * T, T};
    const int lane = G.lane;

    for (;;) {
        if (lane == 0) s_task[g] = atomicAdd(ws.counter, 1);
        G.sync();
        int task = s_task[g];
        G.sync();
        if (task >= ntasks) break;

        if (task < nclip) {
            // a part of the pairs clipped at x[n-1]
            const double sc = group_sum(clip_part_sum<K>(v, task, nclip, G), sm, G);
            if (lane == 0) {
                if constexpr (SCATTER) {
                    if (sc != 0.0) atomicAdd(rhs + (n - 1), sc);
                } else {
                    ws.clip_part[task] = sc;
                    clip_contributor_done(rhs, n, ws, nclip);
                }
            }
            G.sync();
            continue;
        }
        task -= nclip;

        // chunk-major: chunk c of every tile that reaches lag c Cg (tile t
        // spans the lags below n - W t), tiles top first within a chunk
        // (Cg = n: one task per tile)
        int c = 0;
        for (;;) {
            const int cnt = (c * Cg < n) ? min(ntile, (n - c * Cg + W - 1) / W) : 0;
            if (cnt == 0 || task < cnt) break;
            task -= cnt;
            ++c;
        }
        const int tile = task, chunk = c;      // tile 0 is the top one (largest first)
        if (tile >= ntile) continue;
        // generic grids walk rows, not lags: one task per tile there
        const int nct = v.geo ? (n - W * tile + Cg - 1) / Cg : 1;
        if (chunk >= nct) continue;

        const int I = n - W * (tile + 1);
        const int smax = min(I + W - 1, n - 2);
        const int d_begin = nct > 1 ? chunk * Cg : 0;
        const int d_end = nct > 1 ? min(n, d_begin + Cg) : n;
        // scatter: skip empty lag chunks (uniform: every thread reads the same entry)
        if (SCATTER && chunk > 0 && ws.Ld[d_begin] > smax) continue;

        // Per-task exponent shift of the weight numerators: th ~ x_I (r-1) is
        // carried as th 2^St ~ (r-1), so sum rate*th keeps the dynamic range of
        // the reference's w*rate even on grids spanning hundreds of octaves.
        const int St = -ilogb(x[max(I, 0)]);
        agg_tile_accumulate<K, true>(v, I, d_begin, d_end, St, red + g * T, sm, G);

        if (!SCATTER && nct > 1) {
            // store this chunk's slot sums; the tile's last chunk task adds all
            // of them in chunk order and runs the epilogue (nobody waits)
            constexpr int R2 = TileSlots<true>::rows;
            double* cp = ws.cpart + static_cast<size_t>(tile) * agg_chunk_bound(n) * R2;
            if (lane < R2) cp[chunk * R2 + lane] = sm.fin[g][lane];
            G.sync();
            if (lane == 0) {
                __threadfence();
                s_last[g] = (atomicAdd(ws.cticket + tile, 1) == nct - 1);
            }
            G.sync();
            if (!s_last[g]) continue;
            __threadfence();
            if (lane < R2) {
                double acc = 0.0;
                for (int c = 0; c < nct; ++c) acc += __ldcg(cp + c * R2 + lane);
                sm.fin[g][lane] = acc;
            }
            G.sync();
        }

        if (lane < W) {
            const int i = I + lane;
            if (i >= 0) {
                const double birth = agg_tile_birth<true>(v, I, lane, St, sm.fin[g]);
                const bool first = !SCATTER || chunk == 0;
                const double death = first ? agg_death<K>(v, i) : 0.0;
                const double val = birth - death;
                if constexpr (SCATTER) {
                    if (val != 0.0) atomicAdd(rhs + i, val);
                } else if (lane == 0 && I >= 1) {
                    ws.tfirst[tile] = val;
                    first_bin_done(rhs, I, ws, tile);
                } else {
                    rhs[i] = rhs[i] + val;
                    if (i == n - 1) clip_contributor_done(rhs, n, ws, nclip);
                }
            }
        } else if (lane == W && tile >= 1) {
            // carry into bin I+W, the first bin of the tile above
            const double c = agg_tile_carry(v, I, St, sm.fin[g]);
            if constexpr (SCATTER) {
                if (c != 0.0) atomicAdd(rhs + I + W, c);
            } else {
                ws.tcarry[tile - 1] = c;
                first_bin_done(rhs, I + W, ws, tile - 1);
            }
        }
        G.sync();
    }
}

// ---------------------------------------------------------------------------
// lane: persistent CTAs pulling lane-block tasks (agg_lane.cuh) on verified
// geometric grids -- clip tasks first, then (block, lag chunk) tasks largest
// first in the order of the prep's table ws.ltask (the full chunks, then each
// block's last chunk by length, so the last wave holds the shortest tasks).
// Returns at once on other grids (the tile kernel
// launched after it takes them). It needs fewer registers than the tile
// kernel, so more CTAs fit on an SM.
// ---------------------------------------------------------------------------
#ifndef PBE_LANE_CTAS
#define PBE_LANE_CTAS 3
#endif
constexpr int kLaneCtas = PBE_LANE_CTAS;           // CTAs per SM (register budget)

template <int K, bool SCATTER, bool STAGE>
__global__ void __launch_bounds__(kMainThreads, kLaneCtas)
agg_lane_kernel(const double* __restrict__ N, const double* __restrict__ x,
                double* __restrict__ rhs, AggWs ws, int n, int ntasks_lane, int nclip,
                double b0, double bbr, double bsh, int lane_C)
{
    // per-warp slot sums, then the staged windows (16-byte aligned offsets)
    extern __shared__ __align__(128) double lsmem[];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_flag;
    __shared__ int s_task;
    __shared__ double s_wsum[kMainThreads / 32];

    if (ws.mom[5] == 0.0) return;                  // not geometric: the tile kernel runs
    const int tid = threadIdx.x;
    AggCellView v;
    v.x = x; v.Nk = N; v.Hk = ws.h; v.Nj = N; v.Hj = ws.h; v.Aj = N; v.AHj = ws.h;
    v.Fs = (K == 2) ? ws.h : N;
    v.a = ws.a; v.ia = ws.ia; v.inv_dx = ws.inv_dx;
    v.Bd = ws.Bd; v.Sd = ws.Sd; v.Ld = ws.Ld;
    v.n = n;
    v.D0 = ws.counter[1];
    v.geo = true;
    v.b0 = b0; v.bbr = bbr; v.bsh = bsh;
#pragma unroll
    for (int q = 0; q < 5; ++q) v.M[q] = ws.mom[q];

    if (tid == 0) {
        mbar_init(&s_bar, 1);
        s_flag = 0;
    }
    __syncthreads();
    constexpr int kRed = 2 * kLaneWarps * kLaneBins;     // per-warp R, TH of every slot
    const LaneSmem lsm{lsmem, lsmem + kRed, lsmem + kRed + kLaneWinMax,
                       lsmem + kRed + 2 * kLaneWinMax};
    const LaneArgs la{ws.Ncp, ws.xcp, ws.lpart, ws.cticket, ws.counter + 4, lane_C};
    const TileGroup G0{0, tid, kMainThreads};
    unsigned phase = 0;
    for (;;) {
        if (tid == 0) s_task = atomicAdd(ws.counter, 1);
        __syncthreads();
        int task = s_task;
        const int stop = s_flag;
        __syncthreads();
        if (task >= ntasks_lane || stop) break;
        if (task < nclip) {
            // a part of the pairs clipped at x[n-1], summed over the CTA in a fixed order
            double sc = warp_sum(clip_part_sum<K>(v, task, nclip, G0));
            if ((tid & 31) == 0) s_wsum[tid >> 5] = sc;
            __syncthreads();
            if (tid == 0) {
                sc = 0.0;
                for (int w = 0; w < kMainThreads / 32; ++w) sc += s_wsum[w];
                if constexpr (SCATTER) {
                    if (sc != 0.0) atomicAdd(rhs + (n - 1), sc);
                } else {
                    ws.clip_part[task] = sc;
                    clip_contributor_done(rhs, n, ws, nclip);
                }
            }
            __syncthreads();
            continue;
        }
        task -= nclip;
        // largest first (the prep's launch order)
        const int t = __ldg(ws.ltask + 2 * task), c = __ldg(ws.ltask + 2 * task + 1);
        lane_task<K, SCATTER, STAGE>(v, ws, la, rhs, t, c, nclip, lsm, &s_bar, phase, &s_flag);
    }
}

// Threads per tile task. A smaller group keeps fewer partial sums per slot
// (the fixed-order reduction costs 2 (W+1) T FP64 adds per task) but runs
// each task longer; with few tasks per group slot the last wave idles.
// PBE_GB300_AGG_GROUP (32, 64, 128 or 256) overrides the rule.
int agg_group_size(long long ntasks, int num_sms)
{
    static const int forced = []() {
        const char* e = std::getenv("PBE_GB300_AGG_GROUP");
        const int v = e ? std::atoi(e) : 0;
        return (v == 32 || v == 64 || v == 128 || v == 256) ? v : 0;
    }();
    if (forced) return forced;
    const long long per_sm = ntasks / (2LL * num_sms);     // tasks per CTA slot at T = 256
    if (per_sm >= 16) return 64;
    if (per_sm >= 6) return 128;
    return 256;
}

// Group size of chunked gather launches (PBE_GB300_AGG_GROUP overrides as for
// agg_group_size): 32.
int agg_group_size_chunked()
{
    static const int forced = []() {
        const char* e = std::getenv("PBE_GB300_AGG_GROUP");
        const int v = e ? std::atoi(e) : 0;
        return (v == 32 || v == 64 || v == 128 || v == 256) ? v : 0;
    }();
    return forced ? forced : 32;
}

// Pair tasks on geometric grids: 1 = lane blocks with bulk-copy staging of the
// j-side operands (default), 2 = lane blocks reading them through the
// read-only cache, 0 = the tile tasks of every grid. PBE_GB300_AGG_PATH
// ("lane", "lane_ldg", "tile") overrides.
int agg_lane_mode()
{
    static const int mode = []() {
        const char* e = std::getenv("PBE_GB300_AGG_PATH");
        if (!e) return 1;
        if (std::strcmp(e, "tile") == 0) return 0;
        if (std::strcmp(e, "lane_ldg") == 0) return 2;
        return 1;
    }();
    return mode;
}

// Tasks that sum the clipped pairs (about n + q^2 pairs on a grid with q bins
// per octave, more on generic grids), spread over parts of ~1024 lags or rows.
int agg_clip_tasks(int n)
{
    const int c = (n + 1023) / 1024;
    return c < 1 ? 1 : (c > kMaxClipTasks ? kMaxClipTasks : c);
}

// kind: kAggFull = tables + pair kernels (the drop-in calls), kAggTables =
// the FULL prep only, kAggStage = the light prep + pair kernels on a
// workspace whose tables an earlier kAggTables / kAggFull call wrote.
enum { kAggFull = 0, kAggTables = 1, kAggStage = 2 };

template <int K, bool SC>
cudaError_t launch_k(const AggArgs& a, const AggWs& ws, int num_sms, cudaStream_t s, int kind)
{
    const int n = a.n;
    const int nb = agg_prep_blocks(n);
    const int ntile = (n + W - 1) / W;
    const int nclip = agg_clip_tasks(n);
    // cut the tiles' lags into chunks when the tiles alone leave the CTA slots
    // with fewer than 4 tasks each (their costs fall linearly from the top
    // tile down, so the largest would set the kernel's time). Gather adds a
    // tile's chunk sums in order; scatter flushes each chunk with atomics.
    int Cg = n;
    long long ngather = ntile;
    if (n >= 2 && ntile < 4 * 2 * num_sms) {
        const long long lags = static_cast<long long>(ntile) * n -
                               static_cast<long long>(W) * ntile * (ntile - 1) / 2;
        const long long target = static_cast<long long>(kChunkTasks) * 2 *
                                 (num_sms < kChunkMaxSms ? num_sms : kChunkMaxSms);
        long long cg = (lags + target - 1) / target;
        cg = ((cg + 31) / 32) * 32;
        if (cg < kChunkMinLags) cg = kChunkMinLags;
        const long long floor_bound = (n + agg_chunk_bound(n) - 1) / agg_chunk_bound(n);
        if (cg < floor_bound) cg = floor_bound;
        if (cg < n) {
            Cg = static_cast<int>(cg);
            ngather = 0;
            for (int c = 0; static_cast<long long>(c) * Cg < n; ++c) {
                const int cnt = (n - c * Cg + W - 1) / W;
                ngather += cnt < ntile ? cnt : ntile;
            }
        }
    }
    const long long ntasks_ll = ngather + nclip;
    if (ntasks_ll > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int ntasks = static_cast<int>(ntasks_ll);
    // lane-block tasks, taken instead of the tiles when the grid turns out
    // geometric (decided on the device by the prep kernel)
    const int lane_mode = agg_lane_mode();
    const int lane_C = lane_chunk_len(n);
    const long long nlane_ll = lane_mode ? lane_tasks(n, lane_C) + nclip : 0;
    if (nlane_ll > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int ntasks_lane = static_cast<int>(nlane_ll);
    // chunked gather: many tasks of few lags; single warps keep the fixed-order
    // reduction (2 W T adds per task) small next to a chunk's pairs
    const int T = (Cg < n) ? agg_group_size_chunked() : agg_group_size(ntasks, num_sms);
    const long long need = (ntasks + (kMainThreads / T) - 1) / (kMainThreads / T);
    const int grid = static_cast<int>(need < 2LL * num_sms ? need : 2LL * num_sms);
    const size_t smem = sizeof(double) * TileSlots<true>::rows * kMainThreads;
    cudaError_t e = cudaFuncSetAttribute(agg_main_kernel<K, SC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    auto lkern = (lane_mode == 2) ? agg_lane_kernel<K, SC, false> : agg_lane_kernel<K, SC, true>;
    const size_t lsmem = sizeof(double) * (2 * kLaneWarps * kLaneBins + 3 * kLaneWinMax);
    const long long lcap = static_cast<long long>(kLaneCtas) * num_sms;
    const int lgrid = static_cast<int>(ntasks_lane < lcap ? ntasks_lane : lcap);
    if (lane_mode) {
        e = cudaFuncSetAttribute(lkern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(lsmem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(lkern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess) return e;
    }
    if (kind == kAggStage) {
        // counter[2] was left at 0 by the previous prep on this workspace
        agg_prep_kernel<K, false><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, n, ws, a.beta0, a.beta_br,
                                                              a.beta_sh);
    } else {
        e = cudaMemsetAsync(ws.counter, 0, 8 * sizeof(int), s);   // prep's block tickets
        if (e != cudaSuccess) return e;
        agg_prep_kernel<K, true><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, n, ws, a.beta0, a.beta_br,
                                                             a.beta_sh);
        if (kind == kAggTables) return cudaGetLastError();
    }
    const bool prof = g_prof_start && g_prof_stop;
    if (prof) cudaEventRecord(g_prof_start, s);
    if (lane_mode && lgrid > 0)
        lkern<<<lgrid, kMainThreads, lsmem, s>>>(a.N, a.x, a.rhs, ws, n, ntasks_lane, nclip,
                                                 a.beta0, a.beta_br, a.beta_sh, lane_C);
    agg_main_kernel<K, SC><<<grid, kMainThreads, smem, s>>>(a.N, a.x, a.rhs, ws, n, ntile, ntasks,
                                                            nclip, a.beta0, a.beta_br, a.beta_sh,
                                                            T, Cg, ntasks_lane);
    if (prof) cudaEventRecord(g_prof_stop, s);
    return cudaGetLastError();
}

template <bool SC>
cudaError_t dispatch(const AggArgs& a, const AggWs& ws, int num_sms, cudaStream_t s, int kind)
{
    switch (a.kernel) {
    case 0: return launch_k<0, SC>(a, ws, num_sms, s, kind);
    case 1: return launch_k<1, SC>(a, ws, num_sms, s, kind);
    case 2: return launch_k<2, SC>(a, ws, num_sms, s, kind);
    case 3: return launch_k<3, SC>(a, ws, num_sms, s, kind);
    case 4: return launch_k<4, SC>(a, ws, num_sms, s, kind);
    case 5: return launch_k<5, SC>(a, ws, num_sms, s, kind);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace

cudaEvent_t g_prof_start = nullptr;
cudaEvent_t g_prof_stop = nullptr;

cudaError_t agg_launch(const AggArgs& a, bool scatter, void* ws_base, int num_sms, cudaStream_t s)
{
    AggWs ws;
    agg_ws_layout(a.n, static_cast<char*>(ws_base), &ws);
    return scatter ? dispatch<true>(a, ws, num_sms, s, kAggFull)
                   : dispatch<false>(a, ws, num_sms, s, kAggFull);
}

cudaError_t agg_tables_launch(const AggArgs& a, void* ws_base, int num_sms, cudaStream_t s)
{
    AggWs ws;
    agg_ws_layout(a.n, static_cast<char*>(ws_base), &ws);
    return dispatch<false>(a, ws, num_sms, s, kAggTables);
}

cudaError_t agg_stage_launch(const AggArgs& a, bool scatter, void* ws_base, int num_sms,
                             cudaStream_t s)
{
    AggWs ws;
    agg_ws_layout(a.n, static_cast<char*>(ws_base), &ws);
    return scatter ? dispatch<true>(a, ws, num_sms, s, kAggStage)
                   : dispatch<false>(a, ws, num_sms, s, kAggStage);
}

} // namespace pbe_gb300
