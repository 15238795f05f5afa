// =============================================================================
// pbe_internal.cuh -- device helpers and scratch layouts shared by the
// aggregation and breakage kernels of libpbe_gb300 (sm_103a, FP64).
//
// Design notes that the kernels rely on:
//  * GB300 executes FP64 at 2 DFMA/clk/SM (1.2 TFLOP/s measured; FP64 MMA is
//    no faster). Every FP64 instruction on the per-pair path counts, so
//    comparisons of positive doubles are done on their bit patterns (INT pipe)
//    and per-pair transcendental functions are hoisted to per-bin / per-lag
//    tables computed once per call.
//  * Positive IEEE doubles order like their int64 bit patterns.
// =============================================================================
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace pbe_gb300 {

// ---- launch geometry --------------------------------------------------------
constexpr int kTileW        = 12;    // output bins owned by one task (125 regs, no spill)
constexpr int kMainThreads  = 256;   // threads per aggregation task CTA
constexpr int kPrepThreads  = 64;    // per-bin prep kernels: small blocks spread the
                                     // cube roots and divisions over every SM
constexpr int kMaxClipTasks = 32;    // tasks summing the pairs clipped at x[n-1]
constexpr int kRedRows      = 2 * (kTileW + 1);   // R[0..W], TH[0..W]

// A grid is treated as geometric when |log(x_i/x_0) - i*log(r)| <= kGeoTol for
// every i (r fitted from the end points). Then the pivot ratio x_{j+d}/x_j
// equals x_d/x_0 to ~4*kGeoTol, which keeps the lag tables within 1e-13 of
// the per-pair values.
constexpr double kGeoTol = 5e-14;
constexpr int kLagClipAll = 0x3fffffff;   // lag d whose every pair is clipped

// Guard of the reference breakage kernels (src/breakage_kernels.cuh:131, :195).
constexpr double kBreakageNMin = 2.2e-308;

__device__ __forceinline__ long long dbits(double v) { return __double_as_longlong(v); }

// Geometric-progression fit through x_0 and x_{n-1}, for the deviation test
// |ln(x_i/x_0) - i ln r| <= kGeoTol. Computed in log2 with the binary
// exponents split off exactly (x = 2^E m, m in [1, 2)) and the step
// log2(x_{n-1}/x_0)/(n-1) carried as a double-double, so the test resolves
// ~1e-15 whatever the grid spans (a plain log(x_i/x_0) - i*lr already rounds
// by more than kGeoTol once ln(x_i/x_0) passes ~450).
struct GeoFit {
    int E0;          // exponent of x_0
    double f0;       // log2 of the mantissa of x_0
    double s_hi;     // step, high part
    double s_lo;     // step, low part
};

__device__ __forceinline__ GeoFit geo_fit(double x0, double xl, int n)
{
    GeoFit g;
    g.E0 = ilogb(x0);
    g.f0 = log2(scalbn(x0, -g.E0));
    const int El = ilogb(xl);
    const double fl = log2(scalbn(xl, -El));
    const double m = static_cast<double>(n > 1 ? n - 1 : 1);
    const double L_hi = static_cast<double>(El) - static_cast<double>(g.E0);   // exact
    const double L_lo = fl - g.f0;
    g.s_hi = L_hi / m;
    const double r = fma(-g.s_hi, m, L_hi);                // exact remainder
    g.s_lo = (r + L_lo) / m;
    return g;
}

// |ln(x_i / x_0) - i ln r| for the fitted r (natural-log units).
__device__ __forceinline__ double geo_dev(const GeoFit& g, double xi, int i)
{
    const int Ei = ilogb(xi);
    const double fi = log2(scalbn(xi, -Ei));
    const double di = static_cast<double>(i);
    const double p_hi = di * g.s_hi;
    const double p_lo = fma(di, g.s_hi, -p_hi) + di * g.s_lo;
    const double dev2 = ((static_cast<double>(Ei) - static_cast<double>(g.E0)) - p_hi)
                      + ((fi - g.f0) - p_lo);
    return fabs(dev2) * 0.6931471805599453;
}

// v * 2^s for a normal (or zero) double, by adding s to the exponent field:
// three integer instructions instead of an FP64 multiply. s20 = s << 20.
// Zero stays zero; callers keep |v| 2^s inside the normal range.
__device__ __forceinline__ double scale_pow2(double v, int s20)
{
    int hi = __double2hiint(v);
    const int lo = __double2loint(v);
    hi = (hi & 0x7ff00000) ? hi + s20 : hi;
    return __hiloint2double(hi, lo);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Fixed-order block sum (result valid in every thread). sh: >= blockDim/32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh)
{
    const int nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < nw; ++w) r += sh[w];
    return r;
}

// Left bracket lo in [0, n-2] with x[lo] <= v < x[lo+1], for x[0] < v < x[n-1]
// (same result as the reference's binary searches, src/breakage_kernels.cuh:95-105
// and src/aggregation_kernels.cuh:125-132), comparing bit patterns.
__device__ __forceinline__ int bracket_lo(const double* __restrict__ x, int n, double v)
{
    const long long vb = dbits(v);
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (dbits(__ldg(x + mid)) <= vb) lo = mid; else hi = mid;
    }
    return lo;
}

// Same bracket, for a v known to satisfy x[start] <= v < x[n-1]: gallops up
// from start (1, 2, 4, ... pivots), then bisects the last step. One load when
// v < x[start+1], as for most lags of x_0 + x_d on a fine geometric grid.
__device__ __forceinline__ int bracket_from(const double* __restrict__ x, int n, double v,
                                            int start)
{
    const long long vb = dbits(v);
    int lo = start, step = 1;
    while (lo + step < n - 1 && dbits(__ldg(x + lo + step)) <= vb) {
        lo += step;
        step <<= 1;
    }
    int hi = min(lo + step, n - 1);          // x[hi] > v
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (dbits(__ldg(x + mid)) <= vb) lo = mid; else hi = mid;
    }
    return lo;
}

// Same bracket, for a v known to satisfy x[0] < v < x[start+1]: gallops down
// from start (1, 2, 4, ... pivots), then bisects the last step.
__device__ __forceinline__ int bracket_down(const double* __restrict__ x, double v, int start)
{
    const long long vb = dbits(v);
    int hi = start + 1, step = 1;            // x[hi] > v
    while (hi - step > 0 && dbits(__ldg(x + hi - step)) > vb) {
        hi -= step;
        step <<= 1;
    }
    int lo = hi - step > 0 ? hi - step : 0;  // x[lo] <= v
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (dbits(__ldg(x + mid)) <= vb) lo = mid; else hi = mid;
    }
    return lo;
}

// Selection function S(v) (reference src/breakage_kernels.cuh:51-65).
template <int F>
__device__ __forceinline__ double selection(double v, double S0, double v_ref, double alpha,
                                            double v_min)
{
    if constexpr (F == 0) return S0;
    else if constexpr (F == 1) return S0 * v / v_ref;
    else if constexpr (F == 2) return S0 * pow(v / v_ref, alpha);
    else return (v > v_min) ? S0 : 0.0;
}

// Bracket of a fragment volume: -1 when clipped to bin 0 (v <= x[0]), n-1 when
// clipped to bin n-1 (v >= x[n-1]), else lo with x[lo] <= v < x[lo+1].
__device__ __forceinline__ int frag_bracket(const double* __restrict__ x, int n, double v)
{
    if (dbits(v) <= dbits(__ldg(x)) || !(v > 0.0)) return -1;
    if (dbits(v) >= dbits(__ldg(x + n - 1))) return n - 1;
    return bracket_lo(x, n, v);
}

// log2 of a positive normal double in FP32 (exponent from the bits, the
// mantissa's log2 by the SFU): a few 1e-5 absolute, enough to guess an index.
__device__ __forceinline__ float log2_approx(double v)
{
    const long long b = dbits(v);
    const int e = static_cast<int>((b >> 52) & 0x7ff) - 1023;
    const float m = __int_as_float(0x3f800000 | static_cast<int>((b >> 29) & 0x7fffff));   // [1, 2)
    return static_cast<float>(e) + __log2f(m);
}

// frag_bracket, started where a geometric grid through x[0] and x[n-1] would
// put v (lx0 = log2_approx(x[0]), inv_span = (n - 1) / (log2 x[n-1] - lx0)),
// then galloping to the exact bracket: one or two loads on a geometric grid,
// a logarithmic number on any other.
__device__ __forceinline__ int frag_bracket_guess(const double* __restrict__ x, int n, double v,
                                                  float lx0, float inv_span)
{
    if (dbits(v) <= dbits(__ldg(x)) || !(v > 0.0)) return -1;
    if (dbits(v) >= dbits(__ldg(x + n - 1))) return n - 1;
    float gf = (log2_approx(v) - lx0) * inv_span;
    gf = fminf(fmaxf(gf, 0.0f), static_cast<float>(n - 2));
    const int g = static_cast<int>(gf);
    return dbits(__ldg(x + g)) <= dbits(v) ? bracket_from(x, n, v, g) : bracket_down(x, v, g - 1);
}

// frag_bracket of a v at or below a volume whose frag_bracket is `above`.
__device__ __forceinline__ int frag_bracket_below(const double* __restrict__ x, int n, double v,
                                                  int above)
{
    if (above < 0 || dbits(v) <= dbits(__ldg(x)) || !(v > 0.0)) return -1;
    if (dbits(v) >= dbits(__ldg(x + n - 1))) return n - 1;
    return bracket_down(x, v, above < n - 2 ? above : n - 2);
}

// ---- aggregation scratch ----------------------------------------------------
// Pivot volumes enter the weights only through differences v - x_lo. Each task
// carries them shifted by the exponent of its own tile (times 2^St, exact), so
// sum rate*(v - x_lo) neither overflows nor underflows earlier than the
// reference's (1-w)*rate and w*rate would, whatever range the grid spans.
// Pivots must be positive normal doubles.
struct AggWs {
    double* h;         // [n]  x_i N_i
    double* a;         // [n]  x_i^(1/3)
    double* ia;        // [n]  1 / x_i^(1/3)
    double* inv_dx;    // [n]  1 / (x_{i+1} - x_i)   (entry n-1 unused)
    double* Bd;        // [n]  per-lag factor (see agg_prep_kernel)
    double* Sd;        // [n]  per-lag factor multiplying x_j
    int*    Ld;        // [n]  bracket offset of lag d: lo(j, j+d) = j + Ld[d]
    double* mom_part;  // [nb_prep * 8] per-block moment partials
    double* mom;       // [8]  M_{-1/3}, M_0, M_{1/3}, M_{2/3}, M_1, geo flag, max dev
    double* clip_part; // [kMaxClipTasks] sums of clipped pair rates, one per clip task
    double* tfirst;    // [ntile] gather mode: tile's own value of its first bin
    double* tcarry;    // [ntile] gather mode: the lower neighbour's carry into that bin
    int*    tticket;   // [ntile] contributors to the tile's first bin done (0, 1, 2)
    double* cpart;     // [ntile * agg_chunk_bound(n) * 2 kTileW] lag-chunk partials of R, TH
    int*    cticket;   // [ntile] lag-chunk tasks of the tile done
    int*    counter;   // [8]  [0] task counter, [1] first lag with Ld[d] == d,
                       //      [2] prep blocks done, [3] bin n-1 contributors done,
                       //      [4] a staging wait of the lane tasks gave up
    double* Ncp;       // [n + 2] copy of N, 256-byte aligned (bulk-copy source)
    double* xcp;       // [n + 2] copy of x, 256-byte aligned (bulk-copy source)
    double* lpart;     // [lane_partial_doubles(n)] lane-task chunk partials
    int*    ltask;     // [2 lane_tasks(n)] lane tasks in launch order, (block, chunk) pairs
};

constexpr int agg_prep_blocks(int n) { return (n + kPrepThreads - 1) / kPrepThreads; }
__host__ __device__ constexpr int agg_tiles(int n) { return (n + kTileW - 1) / kTileW; }

// Gather mode with few tiles per CTA slot (small n): each tile's lags are cut
// into chunks of at least kChunkMinLags lags, about kChunkTasks tasks per CTA
// slot in all, on GPUs of up to kChunkMaxSms SMs; agg_chunk_bound(n) chunks per
// tile at most (the scratch is sized for it whatever the GPU).
constexpr int kChunkTasks = 8;
constexpr int kChunkMaxSms = 256;
constexpr int kChunkMinLags = 256;
__host__ __device__ constexpr int agg_chunk_bound(int n)
{
    const int a = (n + kChunkMinLags - 1) / kChunkMinLags;
    const int b = n > 0 ? (2 * kTileW * kChunkTasks * 2 * kChunkMaxSms + n - 1) / n + 1 : 1;
    const int m = a < b ? a : b;
    return m < 1 ? 1 : m;
}

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Lane-block pair tasks (agg_lane.cuh): blocks of kLaneBins output bins
// aligned to the top of the grid, cut into lag chunks of lane_chunk_len(n)
// lags (at least n / 16 by default, so at most 17 chunks per block). Task (block t,
// chunk c) has the index sum_{c' < c} lane_chunk_blocks(c') + t; its chunk
// partial (R, TH of 32 slots) is stored under that index.
constexpr int kLaneBins = 32;
#ifndef PBE_LANE_MIN_CHUNK
#define PBE_LANE_MIN_CHUNK 256
#endif
constexpr int kLaneMinChunk = PBE_LANE_MIN_CHUNK;   // shortest lag chunk

__host__ __device__ constexpr int lane_blocks(int n) { return (n + kLaneBins - 1) / kLaneBins; }
// Highest slot of block t (slots exist up to n - 2); < 0 when the block has none.
__host__ __device__ constexpr int lane_block_smax(int n, int t)
{
    return (n - kLaneBins * t - 1) < n - 2 ? (n - kLaneBins * t - 1) : n - 2;
}
// Lag chunk length: at least n / PBE_LANE_CHUNK_DIV (16), a multiple of 64, at
// least kLaneMinChunk. At n = 3840 the chunk lengths 128 to 512 measured
// within 2 % of each other; at n = 16384, 576 to 1408 within 1 %.
#ifndef PBE_LANE_CHUNK_DIV
#define PBE_LANE_CHUNK_DIV 16
#endif
__host__ __device__ constexpr int lane_chunk_len(int n)
{
    const int c = (((n + PBE_LANE_CHUNK_DIV - 1) / PBE_LANE_CHUNK_DIV) + 63) / 64 * 64;
    return c < kLaneMinChunk ? kLaneMinChunk : c;
}
// Chunks of block t: every block has chunk 0; chunk c >= 1 when c C <= smax_t.
__host__ __device__ constexpr int lane_block_chunks(int n, int t, int C)
{
    return lane_block_smax(n, t) < 0 ? 1 : lane_block_smax(n, t) / C + 1;
}
// Blocks that have chunk c (they are blocks 0 .. cnt-1: smax_t falls with t).
__host__ __device__ constexpr int lane_chunk_blocks(int n, int c, int C)
{
    if (c == 0) return lane_blocks(n);
    if (static_cast<long long>(c) * C > n - 2) return 0;
    const long long m = (n - 1 - static_cast<long long>(c) * C) / kLaneBins + 1;
    return m < lane_blocks(n) ? static_cast<int>(m) : lane_blocks(n);
}
__host__ __device__ constexpr long long lane_tasks(int n, int C)
{
    long long s = 0;
    for (int c = 0; lane_chunk_blocks(n, c, C) > 0; ++c) s += lane_chunk_blocks(n, c, C);
    return s;
}
// Launch order of the lane tasks (largest first, so the last wave is filled
// with the shortest tasks): first every chunk that is not its block's last
// (all C lags long), chunk by chunk; then each block's last chunk, longest
// first (ties: lower block first). Entry k of the order is lane_task_at(k).
// Full chunks: chunk c of the blocks that also have chunk c + 1.
__host__ __device__ constexpr int lane_full_tasks(int n, int C)
{
    int s = 0;
    for (int c = 0; lane_chunk_blocks(n, c + 1, C) > 0; ++c) s += lane_chunk_blocks(n, c + 1, C);
    return s;
}
// Lags of block t's last chunk (before the cut where Ld passes its top slot).
__host__ __device__ constexpr int lane_last_chunk_len(int n, int t, int C)
{
    return lane_block_smax(n, t) + 1 - (lane_block_chunks(n, t, C) - 1) * C;
}

// Position of block t's last chunk among the last chunks (longest first, then
// lower block first). For t >= 1 the block's top slot is n - 1 - 32 t, so its
// last chunk has ((n - 33 - 32 (t - 1)) mod C) + 1 lags: blocks whose t - 1
// agree mod P = C / 32 share a length. Counts per class, P steps.
__host__ __device__ inline int lane_last_rank(int n, int t, int C)
{
    const int nblk = lane_blocks(n);
    const int lt = lane_last_chunk_len(n, t, C), l0 = lane_last_chunk_len(n, 0, C);
    const int Lt = lt > 0 ? lt : 0;
    const int L0 = l0 > 0 ? l0 : 0;
    int rank = (L0 > Lt || (L0 == Lt && 0 < t)) ? 1 : 0;
    if (nblk >= 2) {
        const int P = C / kLaneBins;
        const int M = nblk - 2;                  // class u has the blocks 1 + u + P k <= nblk - 1
        int rem = (n - 33) % C;                  // (n - 33 - 32 u) mod C; n >= 33 here
        int q = M / P, rq = M - q * P;           // M - u = q P + rq
        for (int u = 0; u < P && u <= M; ++u) {
            if (rem + 1 > Lt) rank += q + 1;
            rem -= kLaneBins;
            if (rem < 0) rem += C;
            if (--rq < 0) { rq += P; --q; }
        }
        if (t >= 1) rank += (t - 1) / P;         // same length, lower block
    }
    return rank;
}

// Doubles of lane-task chunk partials: tasks x (R, TH) x kLaneBins.
__host__ __device__ constexpr size_t lane_partial_doubles(int n)
{
    return static_cast<size_t>(lane_tasks(n, lane_chunk_len(n))) * 2 * kLaneBins;
}

// Size of the aggregation scratch for n bins, equal to agg_ws_layout(n) below
// (kept in step with it; usable in constant expressions).
constexpr size_t agg_ws_bytes(int n)
{
    const size_t dn = align256(sizeof(double) * static_cast<size_t>(n));
    return 6 * dn + align256(sizeof(int) * static_cast<size_t>(n))
         + align256(sizeof(double) * 8 * static_cast<size_t>(agg_prep_blocks(n)))
         + align256(sizeof(double) * 8)
         + align256(sizeof(double) * kMaxClipTasks)
         + 2 * align256(sizeof(double) * static_cast<size_t>(agg_tiles(n)))
         + align256(sizeof(int) * static_cast<size_t>(agg_tiles(n)))
         + align256(sizeof(double) * 2 * kTileW * static_cast<size_t>(agg_tiles(n)) *
                    static_cast<size_t>(agg_chunk_bound(n)))
         + align256(sizeof(int) * static_cast<size_t>(agg_tiles(n)))
         + align256(sizeof(int) * 8)
         + 2 * align256(sizeof(double) * (static_cast<size_t>(n) + 2))
         + align256(sizeof(double) * lane_partial_doubles(n))
         + align256(sizeof(int) * 2 * static_cast<size_t>(lane_tasks(n, lane_chunk_len(n))));
}

// Carves the aggregation scratch out of `base` (may be null to query the size).
inline size_t agg_ws_layout(int n, char* base, AggWs* ws)
{
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align256(bytes); return p; };
    const size_t dn = sizeof(double) * static_cast<size_t>(n);
    AggWs w{};
    w.h         = reinterpret_cast<double*>(take(dn));
    w.a         = reinterpret_cast<double*>(take(dn));
    w.ia        = reinterpret_cast<double*>(take(dn));
    w.inv_dx    = reinterpret_cast<double*>(take(dn));
    w.Bd        = reinterpret_cast<double*>(take(dn));
    w.Sd        = reinterpret_cast<double*>(take(dn));
    w.Ld        = reinterpret_cast<int*>(take(sizeof(int) * static_cast<size_t>(n)));
    w.mom_part  = reinterpret_cast<double*>(take(sizeof(double) * 8 * static_cast<size_t>(agg_prep_blocks(n))));
    w.mom       = reinterpret_cast<double*>(take(sizeof(double) * 8));
    w.clip_part = reinterpret_cast<double*>(take(sizeof(double) * kMaxClipTasks));
    const size_t nt = static_cast<size_t>(agg_tiles(n));
    w.tfirst    = reinterpret_cast<double*>(take(sizeof(double) * nt));
    w.tcarry    = reinterpret_cast<double*>(take(sizeof(double) * nt));
    w.tticket   = reinterpret_cast<int*>(take(sizeof(int) * nt));
    w.cpart     = reinterpret_cast<double*>(take(sizeof(double) * 2 * kTileW * nt *
                                                 static_cast<size_t>(agg_chunk_bound(n))));
    w.cticket   = reinterpret_cast<int*>(take(sizeof(int) * nt));
    w.counter   = reinterpret_cast<int*>(take(sizeof(int) * 8));
    w.Ncp       = reinterpret_cast<double*>(take(sizeof(double) * (static_cast<size_t>(n) + 2)));
    w.xcp       = reinterpret_cast<double*>(take(sizeof(double) * (static_cast<size_t>(n) + 2)));
    w.lpart     = reinterpret_cast<double*>(take(sizeof(double) * lane_partial_doubles(n)));
    w.ltask     = reinterpret_cast<int*>(take(sizeof(int) * 2 *
                                              static_cast<size_t>(lane_tasks(n, lane_chunk_len(n)))));
    if (ws) *ws = w;
    return off;
}

// ---- breakage scratch (gather mode) ------------------------------------------
// Fragment (q, j) has the bracket lo = -1 (clipped to bin 0), n-1 (clipped to
// bin n-1) or x[lo] <= x_j t_q < x[lo+1].
struct BrkWs {
    double* clo;   // [nq * n]  share of fragment (q, j) deposited at lo (all of it when clipped)
    double* chi;   // [nq * n]  share deposited at lo + 1
    int*    first; // [nq * (n + 2)]  first[q][m+1] = first j with lo(q, j) >= m, m in [-1, n]
    double* SN;    // [n]  S(x_j) N_j (0 where the guard skips bin j)
    double* clipsum; // [nq * n / 256] per prep block: shares clipped below x[0]
    int*    lo;    // [nq * n]  bracket of fragment (q, j) (kept by brk_tables_launch)
    double* Ssel;  // [n]  S(x_j) (kept by brk_tables_launch)
};

inline size_t brk_ws_layout(int n, int nq, char* base, BrkWs* ws)
{
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align256(bytes); return p; };
    const size_t m = static_cast<size_t>(n) * static_cast<size_t>(nq);
    BrkWs w{};
    w.clo   = reinterpret_cast<double*>(take(sizeof(double) * m));
    w.chi   = reinterpret_cast<double*>(take(sizeof(double) * m));
    w.first = reinterpret_cast<int*>(take(sizeof(int) * static_cast<size_t>(nq) * (static_cast<size_t>(n) + 2)));
    w.SN    = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(n)));
    w.clipsum = reinterpret_cast<double*>(take(sizeof(double) * ((m + 255) / 256)));
    w.lo    = reinterpret_cast<int*>(take(sizeof(int) * m));
    w.Ssel  = reinterpret_cast<double*>(take(sizeof(double) * static_cast<size_t>(n)));
    if (ws) *ws = w;
    return off;
}

// ---- VJP scratch ---------------------------------------------------------------
// The single-instance VJP may split each row tile's partner range into up to
// this many chunks (separate tasks) to even out the last wave.
constexpr int kVjpMaxChunks = 8;

// Lane-block VJP tasks on geometric grids (vjp.cu): row block b holds the rows
// [32 b, 32 b + 32) and meets the lags d in [1, n - 1 - 32 b] (partner
// k = j + d), cut into chunks of vjp_lane_chunk(n) lags. Task (b, c) has the
// index sum_{c' < c} vjp_lane_chunk_blocks(c') + b; it stores the 2 x 32 sums
// of its rows as the smaller member and C + 32 sums of the rows
// 32 b + c C + i (i < C + 32) as the larger member.
// Chunk length: at least n / PBE_VJP_CHUNK_DIV lags, a multiple of 64, at least
// kLaneMinChunk. C >= 32: a row then lies in the windows of at most two chunks
// of a block.
#ifndef PBE_VJP_CHUNK_DIV
#define PBE_VJP_CHUNK_DIV 16
#endif
#ifndef PBE_VJP_MIN_CHUNK
#define PBE_VJP_MIN_CHUNK 256
#endif
__host__ __device__ constexpr int vjp_lane_chunk(int n)
{
    const int c = (((n + PBE_VJP_CHUNK_DIV - 1) / PBE_VJP_CHUNK_DIV) + 63) / 64 * 64;
    return c < PBE_VJP_MIN_CHUNK ? PBE_VJP_MIN_CHUNK : c;
}
static_assert(PBE_VJP_MIN_CHUNK >= 32, "vjp lane chunks must be at least 32 lags");
// Row blocks that have chunk c (blocks 0 .. cnt-1: the lag range shrinks with b).
__host__ __device__ constexpr int vjp_lane_chunk_blocks(int n, int c, int C)
{
    const long long r = n - 1 - static_cast<long long>(c) * C;   // lags of block 0 from chunk c on
    return r >= 1 ? static_cast<int>((r - 1) / kLaneBins + 1) : 0;
}
__host__ __device__ constexpr int vjp_lane_chunks(int n, int C)
{
    return n >= 2 ? (n - 2) / C + 1 : 0;
}
__host__ __device__ constexpr long long vjp_lane_tasks(int n, int C)
{
    long long s = 0;
    for (int c = 0; vjp_lane_chunk_blocks(n, c, C) > 0; ++c) s += vjp_lane_chunk_blocks(n, c, C);
    return s;
}
// Launch order (largest first, as the forward's lane tasks): every chunk that is
// not its row block's last, chunk by chunk, then each block's last chunk,
// longest first (ties: lower block first).
__host__ __device__ constexpr int vjp_lane_full_tasks(int n, int C)
{
    int s = 0;
    for (int c = 0; vjp_lane_chunk_blocks(n, c + 1, C) > 0; ++c) s += vjp_lane_chunk_blocks(n, c + 1, C);
    return s;
}
// Position of row block b's last chunk among the last chunks: block b meets
// the lags [1, n - 1 - 32 b], so its last chunk has ((n - 2 - 32 b) mod C) + 1
// lags; blocks that agree mod P = C / 32 share a length.
__host__ __device__ inline int vjp_lane_last_rank(int n, int b, int C)
{
    const int nvb = vjp_lane_chunk_blocks(n, 0, C);     // blocks with at least one lag
    const int P = C / kLaneBins;
    const int r0 = (n - 2) % C;
    int remb = (r0 - kLaneBins * (b % P)) % C;
    if (remb < 0) remb += C;
    const int Lb = remb + 1;
    int rank = b / P;                                   // same length, lower block
    const int M = nvb - 1;                              // class u has the blocks u + P k <= nvb - 1
    int rem = r0;                                       // (r0 - 32 u) mod C
    int q = M / P, rq = M - q * P;                      // M - u = q P + rq
    for (int u = 0; u < P && u <= M; ++u) {
        if (rem + 1 > Lb) rank += q + 1;
        rem -= kLaneBins;
        if (rem < 0) rem += C;
        if (--rq < 0) { rq += P; --q; }
    }
    return rank;
}
struct VjpWs {
    double* h;         // [n]  x_i N_i
    double* a;         // [n]  x_i^(1/3)
    double* ia;        // [n]  1 / x_i^(1/3)
    double* D;         // [n]  (lambda_{i+1} - lambda_i) / (x_{i+1} - x_i)
    double* Bf;        // [n]  Brownian factor of lag d (rho + 1/rho + 2), no beta, no 1/2
    double* Sf;        // [n]  shear factor of lag d (1 + rho)^3 (times x of the smaller member)
    double* Sl;        // [n]  the same times x_0 / x_d: times x of the larger member
    int*    Ld;        // [n]  bracket offset of lag d (as AggWs)
    double* mom_part;  // [nb_prep * 16] moments of N and lambda*N, max deviation
    double* mom;       // [16] 0..4 moments of N, 5..9 of lambda*N, 10 geo flag
    double* gpart;     // [max(ntile, n / 8) * 4] per-task / per-block parameter partials
    double* vpart;     // [ntile * kVjpMaxChunks * 2 kTileW] row sums per (tile, partner chunk)
    int*    ltask;     // [2 lane tasks] lane tasks in launch order, (row block, chunk) pairs
    double* lup;       // [lane tasks * 64] lane-task sums of the rows as smaller members
    double* llo;       // [lane tasks * (C + 32)] lane-task sums of the rows as larger members
    int*    counter;   // [8]: 0 tile tasks, 1 lane tasks
};

inline size_t vjp_ws_layout(int n, char* base, VjpWs* ws)
{
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align256(bytes); return p; };
    const size_t dn = sizeof(double) * static_cast<size_t>(n);
    const int ntile = (n + kTileW - 1) / kTileW;
    const int nbb = (n + 7) / 8;          // breakage VJP blocks: 256 / 32 parents at least
    VjpWs w{};
    w.h        = reinterpret_cast<double*>(take(dn));
    w.a        = reinterpret_cast<double*>(take(dn));
    w.ia       = reinterpret_cast<double*>(take(dn));
    w.D        = reinterpret_cast<double*>(take(dn));
    w.Bf       = reinterpret_cast<double*>(take(dn));
    w.Sf       = reinterpret_cast<double*>(take(dn));
    w.Sl       = reinterpret_cast<double*>(take(dn));
    w.Ld       = reinterpret_cast<int*>(take(sizeof(int) * static_cast<size_t>(n)));
    w.mom_part = reinterpret_cast<double*>(take(sizeof(double) * 16 * static_cast<size_t>(agg_prep_blocks(n))));
    w.mom      = reinterpret_cast<double*>(take(sizeof(double) * 16));
    w.gpart    = reinterpret_cast<double*>(take(sizeof(double) * 4 * static_cast<size_t>(ntile > nbb ? ntile : nbb)));
    w.vpart    = reinterpret_cast<double*>(take(sizeof(double) * 2 * kTileW * kVjpMaxChunks *
                                                static_cast<size_t>(ntile)));
    const int C = vjp_lane_chunk(n);
    const size_t ltasks = static_cast<size_t>(vjp_lane_tasks(n, C));
    w.ltask    = reinterpret_cast<int*>(take(sizeof(int) * 2 * ltasks));
    w.lup      = reinterpret_cast<double*>(take(sizeof(double) * 2 * kLaneBins * ltasks));
    w.llo      = reinterpret_cast<double*>(take(sizeof(double) * (C + 32) * ltasks));
    w.counter  = reinterpret_cast<int*>(take(sizeof(int) * 8));
    if (ws) *ws = w;
    return off;
}

struct AggVjpArgs {
    const double* N; const double* x; const double* lam; double* gN; double* gp;
    int n; int kernel; double beta0, beta_br, beta_sh;
};
struct BrkVjpArgs {
    const double* N; const double* x; const double* t_q; const double* bw_q; const double* lam;
    double* gN; double* gp;
    int n; int n_quad; int selection; double S0, v_ref, alpha, v_min;
};
cudaError_t agg_vjp_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s);
// For callers that keep a VJP workspace per set of pivots (the RK4 tape):
// agg_vjp_tables_launch writes the grid-only tables (cube roots, lag tables,
// bracket offsets, geometric flag); agg_vjp_stage_launch then runs the VJP for
// any N and lambda on that workspace, with the result of agg_vjp_launch.
cudaError_t agg_vjp_tables_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s);
cudaError_t agg_vjp_stage_launch(const AggVjpArgs& a, void* ws_base, int num_sms, cudaStream_t s);
// Ssel / lo_tab (nullable): the selection function per bin and the fragment
// brackets [q n + j] of a breakage table workspace (brk_tables_launch) for the
// same pivots, quadrature and parameters; the kernel then skips their
// computation (same values).
cudaError_t brk_vjp_launch(const BrkVjpArgs& a, void* ws_base, cudaStream_t s,
                           const double* Ssel = nullptr, const int* lo_tab = nullptr);

// ---- profiling hook ----------------------------------------------------------
// When both are non-null the aggregation launcher records g_prof_start right
// before and g_prof_stop right after its main (pair) kernel, on the call's
// stream. Set through pbe_set_profile_events(); process-wide, not thread-safe.
extern cudaEvent_t g_prof_start;
extern cudaEvent_t g_prof_stop;

// ---- host-side launchers (defined in aggregation.cu / breakage.cu) ----------
struct AggArgs {
    const double* N; const double* x; double* rhs;
    int n; int kernel; double beta0, beta_br, beta_sh;
};
struct BrkArgs {
    const double* N; const double* x; const double* t_q; const double* bw_q; double* rhs;
    int n; int n_quad; int selection; double S0, v_ref, alpha, v_min;
};

// true when `mode` (PBE_MODE_*) resolves to the scatter variant. Defined in api.cu.
bool mode_is_scatter(int mode);

// Launch the aggregation kernels with a scratch buffer `ws_base` of at least
// agg_ws_layout(n) bytes. scatter selects the atomic-flush variant.
cudaError_t agg_launch(const AggArgs& a, bool scatter, void* ws_base, int num_sms, cudaStream_t s);
// For callers that keep a workspace per (pivots, coefficients) -- the RK4
// tape: agg_tables_launch writes the grid-only tables (cube roots, 1/dx, lag
// tables, geometric flag, D0) into it; agg_stage_launch then evaluates the
// RHS for any N on that workspace, recomputing only what depends on N, and
// gives bitwise the result of agg_launch.
cudaError_t agg_tables_launch(const AggArgs& a, void* ws_base, int num_sms, cudaStream_t s);
cudaError_t agg_stage_launch(const AggArgs& a, bool scatter, void* ws_base, int num_sms,
                             cudaStream_t s);
// Breakage: scatter needs no scratch (ws_base may be null).
cudaError_t brk_launch(const BrkArgs& a, bool scatter, void* ws_base, cudaStream_t s);
// Gather mode on a kept workspace (the RK4 tape): brk_tables_launch writes the
// grid-only tables (fragment brackets and run starts, the selection function
// per bin) for the pivots, quadrature table and selection parameters;
// brk_stage_launch then evaluates the RHS for any N on that workspace with
// bitwise the result of brk_launch in gather mode.
cudaError_t brk_tables_launch(const BrkArgs& a, void* ws_base, cudaStream_t s);
cudaError_t brk_stage_launch(const BrkArgs& a, void* ws_base, cudaStream_t s);

} // namespace pbe_gb300
