// =============================================================================
// agg_tile.cuh -- the aggregation tile task, shared by the single-instance
// kernel (aggregation.cu) and the batched-cell kernel (batch_kernels.cu).
//
// A tile task owns the kTileW output bins [I, I + kTileW) of one cell and
// accumulates, for its slots s, R_s = sum of the rates of the pairs whose
// bracket is lo = s and TH_s = sum rate * (v - x_s) 2^St
// (reference: src/aggregation_kernels.cuh:145-239, regrouped; the file header
// of aggregation.cu gives the derivation). A task runs on a "group" of T
// threads (T = 32, 64, 128 or 256, a runtime value) synchronised by a named
// barrier, so one CTA can work on up to eight small tiles at once.
//
// The cell is described by AggCellView. Its j-side arrays (Nj, Hj) may carry
// the cell's kernel coefficient already (batched use, where the per-lag tables
// are shared by every cell on the same grid and hold no beta); the k-side
// arrays (Nk, Hk) and the per-slot factor Fs are plain N and x N.
// =============================================================================
#pragma once

#include "pbe_internal.cuh"
#include "exact_weight.cuh"

namespace pbe_gb300 {

template <int K> struct NeedH {
    static constexpr bool j = (K == 1 || K == 2 || K == 4 || K == 5);
    static constexpr bool k = (K == 1 || K == 2);
};

// Pair rate on a verified geometric grid, lag tables B = c_d * Bfactor(d),
// S = c_d * Sfactor(d) with c_d = 1/2 for d = 0 (times beta in the
// single-instance tables; the batched tables leave beta to Nj / Hj).
template <int K>
__device__ __forceinline__ double rate_geo(double B, double S, double Nj, double hj,
                                           double Nk, double hk)
{
    if constexpr (K == 0 || K == 3) return (B * Nj) * Nk;
    else if constexpr (K == 1) return B * fma(hj, Nk, Nj * hk);
    else if constexpr (K == 2) return (B * hj) * hk;
    else if constexpr (K == 4) return (S * hj) * Nk;
    else return Nk * fma(S, hj, B * Nj);
}

// Lags whose pairs land on the larger member's own slot (lo = k): the rate is
// F_k * q_slot(j) with the per-slot factor F_k = N_k (h_k for Product). Not
// used for Sum, whose rate has two k-dependent terms.
template <int K>
__device__ __forceinline__ double q_slot(double B, double S, double Nj, double hj)
{
    if constexpr (K == 0 || K == 3) return B * Nj;
    else if constexpr (K == 2) return B * hj;
    else if constexpr (K == 4) return S * hj;
    else return fma(S, hj, B * Nj);
}

// Pair rate on any grid from per-bin values (a = x^(1/3), ia = 1/a, h = x N):
// beta of src/aggregation_kernels.cuh:56-89 with the divisions replaced by
// products with the reciprocal cube roots.
template <int K>
__device__ __forceinline__ double rate_gen(bool diag, double b0, double bbr, double bsh,
                                           double Nj, double hj, double aj, double iaj,
                                           double Nk, double hk, double ak, double iak)
{
    double r;
    if constexpr (K == 0) r = (b0 * Nj) * Nk;
    else if constexpr (K == 1) r = b0 * fma(hj, Nk, Nj * hk);
    else if constexpr (K == 2) r = (b0 * hj) * hk;
    else {
        double beta = 0.0;
        if constexpr (K == 3 || K == 5) beta = bbr * (fma(aj, iak, ak * iaj) + 2.0);
        if constexpr (K == 4 || K == 5) { const double s = aj + ak; beta = fma(bsh * s, s * s, beta); }
        r = (beta * Nj) * Nk;
    }
    return diag ? 0.5 * r : r;
}

// sum_k beta(x_i, x_k) N_k from the moments
// M[0] = sum N/a, M[1] = sum N, M[2] = sum a N, M[3] = sum a^2 N, M[4] = sum x N.
template <int K>
__device__ __forceinline__ double death_factor(double xi, double ai, double iai,
                                               const double* M, double b0, double bbr,
                                               double bsh)
{
    if constexpr (K == 0) return b0 * M[1];
    else if constexpr (K == 1) return b0 * fma(xi, M[1], M[4]);
    else if constexpr (K == 2) return (b0 * xi) * M[4];
    else {
        double f = 0.0;
        // beta_br (a_i/a_k + a_k/a_i + 2)
        if constexpr (K == 3 || K == 5) f = bbr * (fma(ai, M[0], iai * M[2]) + 2.0 * M[1]);
        // beta_sh (a_i + a_k)^3 = beta_sh (x_i + 3 a_i^2 a_k + 3 a_i a_k^2 + x_k)
        if constexpr (K == 4 || K == 5)
            f = fma(bsh, fma(xi, M[1], (3.0 * ai) * fma(ai, M[2], M[3])) + M[4], f);
        return f;
    }
}

// One cell as seen by a tile task.
struct AggCellView {
    const double* x;       // pivots [n]
    const double* Nk;      // N [n]: k side, death, generic path
    const double* Hk;      // x N [n] (K = 1, 2 and the generic path of those)
    const double* Nj;      // j-side N factor [n]
    const double* Hj;      // j-side x N factor [n]
    const double* Aj;      // j-side N, no coefficient [n] (generic path, clipped pairs): N,
                           // or the first vector of a Jacobian-vector pass
    const double* AHj;     // x Aj [n] (K = 1, 2 on the generic path)
    const double* Fs;      // per-slot factor of lo = k lags [n]: N (x N for K = 2)
    const double* a;       // x^(1/3) [n]
    const double* ia;      // x^(-1/3) [n]
    const double* inv_dx;  // 1/(x_{i+1} - x_i) [n]
    const double* Bd;      // per-lag tables [n] (geometric grids)
    const double* Sd;
    const int*    Ld;
    int n;
    int D0;                // first lag with Ld[d] == d
    bool geo;
    double b0, bbr, bsh;   // kernel coefficients (generic path, death)
    double M[5];           // moments of N (see death_factor)
};

constexpr int kMaxGroups = kMainThreads / 32;

// Slots of a tile task. Without carry: s = I-1 .. I+W-1, slot I-1 feeding only
// the w-part of bin I, so every pair on a tile boundary is evaluated by both
// tiles. With carry: s = I .. I+W-1; the w-part of slot I+W-1 leaves the task
// as a carry into bin I+W, which the neighbour tile combines.
template <bool CARRY> struct TileSlots {
    static constexpr int first = CARRY ? 0 : -1;        // slot t is s = I + first + t
    static constexpr int count = CARRY ? kTileW : kTileW + 1;
    static constexpr int rows = 2 * count;              // R[0..count), TH[0..count)
};

// Static shared memory of a CTA running tile tasks (per group g < kMaxGroups).
struct TileShared {
    double xs[kMaxGroups][kTileW + 2];    // x of the task's slots and of the pivot above
    double fs[kMaxGroups][kTileW + 2];    // per-slot factor
    double part[kMaxGroups][kRedRows];    // 32-column chunk partials (chunk index g*T/32 + c)
    double fin[kMaxGroups][kRedRows];     // R and TH of the task's slots
    double wsum[kMaxGroups];              // per-warp partials of group sums
    double extra[kMaxGroups][kTileW];     // per-bin additions (batched breakage)
    double cinfo[kMaxGroups][8];          // per-task cell values for the epilogue (batched)
    int last[kMaxGroups];                 // this group ran a tile's last lag chunk (batched)
};

// A group of T threads (T a multiple of 32, T <= kMainThreads) working on one
// task; named barrier g + 1 (barrier 0 stays free for __syncthreads).
struct TileGroup {
    int g;       // group index within the CTA
    int lane;    // thread index within the group
    int T;       // group size
    __device__ __forceinline__ void sync() const
    {
        asm volatile("bar.sync %0, %1;" :: "r"(g + 1), "r"(T) : "memory");
    }
};

// Fixed-order sum over the group (valid in every thread of the group).
__device__ __forceinline__ double group_sum(double v, TileShared& sm, const TileGroup& G)
{
    v = warp_sum(v);
    const int nw = G.T >> 5, wb = G.g * nw;
    G.sync();
    if ((G.lane & 31) == 0) sm.wsum[wb + (G.lane >> 5)] = v;
    G.sync();
    double r = 0.0;
    for (int w = 0; w < nw; ++w) r += sm.wsum[wb + w];
    return r;
}

// Accumulates R_s, TH_s of the task's slots over the lags [d_begin, d_end)
// (geometric grid) or over every row (generic grid) into sm.fin[G.g].
// red: this group's first column of the CTA's kRedRows x kMainThreads
// reduction buffer (row stride kMainThreads). St: exponent shift of the
// weight numerators (-ilogb(x[max(I, 0)])). I may be negative (a tile whose
// lowest bins lie below bin 0).
template <int K, bool CARRY>
__device__ __forceinline__ void agg_tile_accumulate(const AggCellView& v, int I, int d_begin,
                                                    int d_end, int St, double* red,
                                                    TileShared& sm, const TileGroup& G)
{
    constexpr int W = kTileW;
    constexpr int NS = TileSlots<CARRY>::count;
    constexpr int RS = kMainThreads;     // row stride of red
    const int n = v.n;
    const int lane = G.lane, T = G.T;
    const int base = I + TileSlots<CARRY>::first;   // slot of t = 0
    const int smax = min(I + W - 1, n - 2);     // highest non-clipped slot
    double* xs = sm.xs[G.g];
    double* fs = sm.fs[G.g];
    if (lane < NS + 1) {
        const int s = base + lane;
        const bool in = (s >= 0 && s < n);
        xs[lane] = in ? v.x[s] : 0.0;
        fs[lane] = in ? v.Fs[s] : 0.0;
    }
    const int St20 = St << 20;
    G.sync();

    if (v.geo) {
        double R[NS], TH[NS];
#pragma unroll
        for (int t = 0; t < NS; ++t) { R[t] = 0.0; TH[t] = 0.0; }
        const int thi = smax - base;      // slot index t <= thi
        // lags d >= D0 put every pair on its larger member's own slot (lo = k)
        const int D0 = (K == 1) ? n : v.D0;
        const double* __restrict__ Nj_ = v.Nj;
        const double* __restrict__ Hj_ = v.Hj;
        const double* __restrict__ Nk_ = v.Nk;
        const double* __restrict__ Hk_ = v.Hk;
        const double* __restrict__ x_ = v.x;
        int d = d_begin + lane;
        // phase 1, lags with lo > k: rate per pair, R += rate, TH += rate * th
        for (; d < d_end && d < D0; d += T) {
            const int L = __ldg(v.Ld + d);
            if (L > smax) { d = d_end; break; }   // Ld is nondecreasing in d
            const double B = __ldg(v.Bd + d), S = __ldg(v.Sd + d);
            const int jb = base - L;       // j of slot t is jb + t, k = jb + d + t
            const int tlo = max(0, -jb);
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                if (t >= tlo && t <= thi) {
                    const int j = jb + t, k = j + d;
                    const double Nj = __ldg(Nj_ + j), Nk = __ldg(Nk_ + k);
                    const double hj = NeedH<K>::j ? __ldg(Hj_ + j) : 0.0;
                    const double hk = NeedH<K>::k ? __ldg(Hk_ + k) : 0.0;
                    const double rate = rate_geo<K>(B, S, Nj, hj, Nk, hk);
                    // (fl(x_j + x_k) - x_lo) 2^St on the integer pipe, bit-identical
                    // to the reference's two FP64 additions
                    const double th = sum_minus_scaled(__ldg(x_ + k), __ldg(x_ + j), xs[t], St);
                    if (CARRY || t > 0) R[t] += rate;
                    TH[t] = fma(rate, th, TH[t]);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < NS; ++t) {
            red[t * RS + lane] = R[t];
            red[(NS + t) * RS + lane] = TH[t];
            R[t] = 0.0;
            TH[t] = 0.0;
        }
        // phase 2, lags with lo = k: k is the slot itself, so rate = F_slot * q(j)
        // (F = N, or h for Product); sum q and q * th, multiply by F once
        if constexpr (K != 1) {
            for (; d < d_end; d += T) {
                const int L = __ldg(v.Ld + d);
                if (L > smax) break;
                const double B = __ldg(v.Bd + d), S = __ldg(v.Sd + d);
                const int jb = base - L;
                const int tlo = max(0, -jb);
#pragma unroll
                for (int t = 0; t < NS; ++t) {
                    if (t >= tlo && t <= thi) {
                        const int j = jb + t;
                        const double Nj = __ldg(Nj_ + j);
                        const double hj = NeedH<K>::j ? __ldg(Hj_ + j) : 0.0;
                        const double q = q_slot<K>(B, S, Nj, hj);
                        const double th = sum_minus_scaled(xs[t], __ldg(x_ + j), xs[t], St);
                        if (CARRY || t > 0) R[t] += q;
                        TH[t] = fma(q, th, TH[t]);
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                double* r0 = red + t * RS + lane;
                double* r1 = red + (NS + t) * RS + lane;
                *r0 = fma(fs[t], R[t], *r0);
                *r1 = fma(fs[t], TH[t], *r1);
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < 2 * NS; ++r) red[r * RS + lane] = 0.0;
        const int s_first = max(base, 0);
        if (smax >= s_first) {
            const int t_first = s_first - base;
            const int t_last = smax - base;
            const long long blo = dbits(xs[t_first]);
            const long long bhi = dbits(xs[t_last + 1]);
            const double* __restrict__ xsc = v.x;
            const double xlast = xsc[n - 1];
            for (int j = lane; j <= smax; j += T) {
                const double xj = xsc[j];
                if (dbits(xj + xj) >= bhi) break;          // v >= 2 x_j grows with j
                if (dbits(xj + xlast) < blo) continue;     // this row never reaches the tile
                int lo = j, hi = n - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (dbits(xj + xsc[mid]) >= blo) hi = mid; else lo = mid + 1;
                }
                const int ka = lo;
                hi = n;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (dbits(xj + xsc[mid]) >= bhi) hi = mid; else lo = mid + 1;
                }
                const int kb = lo;
                if (ka >= kb) continue;
                const double Nj = v.Aj[j], hj = v.AHj[j], aj = v.a[j], iaj = v.ia[j];
                int t = t_first;
                double Rc = 0.0, THc = 0.0;
                for (int k = ka; k < kb; ++k) {
                    const double vs = xj + xsc[k];
                    const long long vb = dbits(vs);
                    while (t < t_last && dbits(xs[t + 1]) <= vb) {
                        red[t * RS + lane] += Rc;
                        red[(NS + t) * RS + lane] += THc;
                        Rc = 0.0; THc = 0.0; ++t;
                    }
                    const double rate = rate_gen<K>(j == k, v.b0, v.bbr, v.bsh, Nj, hj, aj, iaj,
                                                    v.Nk[k], v.Hk[k], v.a[k], v.ia[k]);
                    Rc += rate;
                    THc = fma(rate, scale_pow2(vs - xs[t], St20), THc);
                }
                red[t * RS + lane] += Rc;
                red[(NS + t) * RS + lane] += THc;
            }
        }
    }
    G.sync();

    // fixed-order reduction: each row in 32-column chunks (the column order
    // rotated by the worker's lane so the chunk reads hit distinct banks),
    // then the chunks of a row in order
    const int nch = T >> 5;
    if (lane < 2 * NS * nch) {
        const int r = lane / nch, c = lane - r * nch;
        const double* p = red + r * RS + c * 32;
        const int rot = lane & 31;
        double s = 0.0;
#pragma unroll 8
        for (int q = 0; q < 32; ++q) s += p[(q + rot) & 31];
        sm.part[G.g * nch + c][r] = s;
    }
    G.sync();
    if (lane < 2 * NS) {
        double s = 0.0;
        for (int c = 0; c < nch; ++c) s += sm.part[G.g * nch + c][lane];
        sm.fin[G.g][lane] = s;
    }
    G.sync();
}

// Birth of bin i = I + t (0 <= i < n) from the task's slot sums (TH carried
// times 2^St). With carry, bin I lacks the w-part of slot I-1 (the lower
// neighbour's carry).
template <bool CARRY>
__device__ __forceinline__ double agg_tile_birth(const AggCellView& v, int I, int t, int St,
                                                 const double* fin)
{
    constexpr int NS = TileSlots<CARRY>::count;
    constexpr int o = -TileSlots<CARRY>::first;        // slot index of bin I
    const int i = I + t;
    double birth = 0.0;
    if (i <= v.n - 2)
        birth = fma(-fin[NS + t + o], scalbn(v.inv_dx[i], -St), fin[t + o]);
    if (i >= 1 && (!CARRY || t >= 1))
        birth = fma(fin[NS + t + o - 1], scalbn(v.inv_dx[i - 1], -St), birth);
    return birth;
}

// With carry: the w-part of slot I+W-1, owed to bin I+W (0 when that slot is
// clipped, i.e. bin I+W does not exist or is bin n-1's own clip slot).
__device__ __forceinline__ double agg_tile_carry(const AggCellView& v, int I, int St,
                                                 const double* fin)
{
    constexpr int NS = TileSlots<true>::count;
    const int s = I + kTileW - 1;
    return (s >= 0 && s <= v.n - 2) ? fin[NS + kTileW - 1] * scalbn(v.inv_dx[s], -St) : 0.0;
}

template <int K>
__device__ __forceinline__ double agg_death(const AggCellView& v, int i)
{
    return v.Nk[i] * death_factor<K>(v.x[i], v.a[i], v.ia[i], v.M, v.b0, v.bbr, v.bsh);
}

} // namespace pbe_gb300
