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
//  * Pairs clipped at x[n-1] are summed by a separate kernel (per lag on a
//    geometric grid, per row otherwise).
//
// Kernels per call: prep (per-bin values, lag tables, moment partials,
// geometric check) -> fin (one block: moments, flag, counter reset) -> clip ->
// main (persistent CTAs pulling target tiles from an atomic counter, largest
// first). GATHER mode: one CTA owns each output bin and reduces it in a fixed
// order -> bitwise reproducible. SCATTER mode: geometric tasks are (tile, lag
// chunk) and flush with FP64 atomicAdd.
// =============================================================================
#include "pbe_internal.cuh"
#include "exact_weight.cuh"

namespace pbe_gb300 {
namespace {

constexpr int W = kTileW;

template <int K> struct NeedH {
    static constexpr bool j = (K == 1 || K == 2 || K == 4 || K == 5);
    static constexpr bool k = (K == 1 || K == 2);
};

// Pair rate on a verified geometric grid, lag tables B = c_d * Bfactor(d),
// S = c_d * Sfactor(d) with c_d = 1/2 for d = 0 (see agg_prep_kernel).
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

// ---------------------------------------------------------------------------
// prep: one thread per bin i. Per-bin values, the lag tables for d = i,
// moment partials and the geometric-grid deviation.
//   Bd[d], Sd[d]: beta(x_j, x_{j+d}) = Bd + x_j Sd on a geometric grid, times
//   c_d (1/2 for d = 0), with rho = x_d^(1/3) / x_0^(1/3):
//     Constant/Sum/Product: Bd = c_d beta0 (the x dependence stays per pair)
//     Brownian: Bd = c_d beta_br (rho + 1/rho + 2)
//     Shear:    Sd = c_d beta_sh (1 + rho)^3
//   Ld[d]: bracket of x_0 + x_d (kLagClipAll when it reaches x[n-1]).
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(kPrepThreads)
agg_prep_kernel(const double* __restrict__ N, const double* __restrict__ x, int n, AggWs ws,
                double b0, double bbr, double bsh)
{
    __shared__ double sh[kPrepThreads / 32];
    __shared__ int d0_s;
    const int i = blockIdx.x * kPrepThreads + threadIdx.x;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double dev = 0.0;
    int d0 = n;      // this thread's lag if its pairs land on their larger member (Ld == d)
    if (threadIdx.x == 0) d0_s = n;
    __syncthreads();
    if (i < n) {
        const double xi = x[i], Ni = N[i];
        const double hi = xi * Ni;
        const double ai = cbrt(xi);
        const double iai = 1.0 / ai;
        ws.h[i] = hi;
        ws.a[i] = ai;
        ws.ia[i] = iai;
        ws.inv_dx[i] = (i < n - 1) ? 1.0 / (x[i + 1] - xi) : 0.0;
        m[0] = iai * Ni; m[1] = Ni; m[2] = ai * Ni; m[3] = (ai * ai) * Ni; m[4] = hi;

        const double x0 = x[0];
        const double c = (i == 0) ? 0.5 : 1.0;
        double B = 0.0, S = 0.0;
        if constexpr (K <= 2) B = c * b0;
        if constexpr (K >= 3) {
            const double rho = ai / cbrt(x0);
            if constexpr (K == 3 || K == 5) B = c * bbr * (rho + 1.0 / rho + 2.0);
            if constexpr (K == 4 || K == 5) { const double s = 1.0 + rho; S = c * bsh * (s * s) * s; }
        }
        ws.Bd[i] = B;
        ws.Sd[i] = S;
        const double v = x0 + xi;
        const int L = (dbits(v) >= dbits(x[n - 1])) ? kLagClipAll : bracket_lo(x, n, v);
        ws.Ld[i] = L;
        if (L == i) d0 = i;
        if (n >= 2) {
            const double lr = log(x[n - 1] / x0) / static_cast<double>(n - 1);
            dev = fabs(log(xi / x0) - static_cast<double>(i) * lr);
            if (!(dev == dev)) dev = 1.0;   // NaN -> not geometric
        }
    }
    atomicMin(&d0_s, d0);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const double s = block_sum(m[q], sh);
        if (threadIdx.x == 0) ws.mom_part[blockIdx.x * 8 + q] = s;
    }
    dev = warp_max(dev);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dev;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < kPrepThreads / 32; ++w) mx = fmax(mx, sh[w]);
        ws.mom_part[blockIdx.x * 8 + 5] = mx;
        ws.mom_part[blockIdx.x * 8 + 6] = static_cast<double>(d0_s);
    }
}

// fin: one block. Moments (fixed-order sums), geometric flag, the first lag
// whose pairs land on their larger member's own slot (Ld[d] == d), counter reset.
__global__ void __launch_bounds__(256) agg_fin_kernel(const double* __restrict__ x, int n, AggWs ws)
{
    __shared__ double sh[8];
    __shared__ int d0_s;
    const int nb = (n + kPrepThreads - 1) / kPrepThreads;
    if (threadIdx.x == 0) d0_s = n;
    __syncthreads();
    int d0 = n;      // smallest lag with Ld[d] == d over the prep blocks
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        d0 = min(d0, static_cast<int>(ws.mom_part[b * 8 + 6]));
    atomicMin(&d0_s, d0);
    for (int q = 0; q < 5; ++q) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) s += ws.mom_part[b * 8 + q];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) ws.mom[q] = s;
    }
    double mx = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) mx = fmax(mx, ws.mom_part[b * 8 + 5]);
    mx = warp_max(mx);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < 8; ++w) mx = fmax(mx, sh[w]);
        // neighbour ratio <= 64 keeps fl(x_j + x_k) within kMaxExpGap binades
        // of its bracket pivot (precondition of sum_minus_scaled)
        const bool ratio_ok = n >= 2 && x[1] <= 64.0 * x[0];
        ws.mom[5] = (n >= 2 && mx <= kGeoTol && ratio_ok) ? 1.0 : 0.0;
        ws.mom[6] = mx;
        ws.counter[0] = 0;
        ws.counter[1] = d0_s;     // lags d >= counter[1] have lo(j, j+d) = j + d
    }
}

// clip: sum of rates of the pairs with x_j + x_k >= x[n-1] (all deposited on
// bin n-1, src/aggregation_kernels.cuh:191-192). One warp per lag d on a
// geometric grid (pairs j in [n-1-Ld, n-1-d]); one warp per row j otherwise
// (k from the first clipped column to n-1).
template <int K, bool SCATTER>
__global__ void __launch_bounds__(kClipWarps * 32)
agg_clip_kernel(const double* __restrict__ N, const double* __restrict__ x, double* rhs,
                int n, AggWs ws, double b0, double bbr, double bsh)
{
    __shared__ double sh[kClipWarps];
    const bool geo = ws.mom[5] != 0.0;
    const int w = blockIdx.x * kClipWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    if (w < n) {
        if (geo) {
            const int d = w;
            const int L = ws.Ld[d];
            const int jhi = n - 1 - d;
            const int jlo = (L >= kLagClipAll) ? 0 : max(0, n - 1 - L);
            const double B = ws.Bd[d], S = ws.Sd[d];
            for (int j = jlo + lane; j <= jhi; j += 32) {
                const double hj = NeedH<K>::j ? ws.h[j] : 0.0;
                const double hk = NeedH<K>::k ? ws.h[j + d] : 0.0;
                acc += rate_geo<K>(B, S, N[j], hj, N[j + d], hk);
            }
        } else {
            const int j = w;
            const double xj = x[j];
            const long long tb = dbits(x[n - 1]);
            int lo = j, hi = n - 1;   // xj + x[n-1] >= x[n-1] always holds
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (dbits(xj + x[mid]) >= tb) hi = mid; else lo = mid + 1;
            }
            const double Nj = N[j], hj = ws.h[j], aj = ws.a[j], iaj = ws.ia[j];
            for (int k = lo + lane; k < n; k += 32)
                acc += rate_gen<K>(j == k, b0, bbr, bsh, Nj, hj, aj, iaj, N[k], ws.h[k], ws.a[k], ws.ia[k]);
        }
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        if constexpr (SCATTER) { if (s != 0.0) atomicAdd(rhs + (n - 1), s); }
        else ws.clip_part[blockIdx.x] = s;
    }
}

// ---------------------------------------------------------------------------
// main: persistent CTAs; each task owns the W bins [I, I+W) of one tile and
// accumulates the slots s = I-1 .. I+W-1 (slot I-1 only feeds the w-part of
// bin I). Thread-private partial sums are reduced in a fixed order.
// ---------------------------------------------------------------------------
template <int K, bool SCATTER>
__global__ void __launch_bounds__(kMainThreads, 2)
agg_main_kernel(const double* __restrict__ N, const double* __restrict__ x,
                double* __restrict__ rhs, AggWs ws, int n, int ntile, int nchunk,
                int ntasks, double b0, double bbr, double bsh)
{
    extern __shared__ double red[];               // [kRedRows][kMainThreads]
    __shared__ double xs[W + 2];                  // x[I-1 .. I+W]
    __shared__ double fs[W + 2];                  // per-slot factor N (h for Product)
    __shared__ double part4[4][kRedRows];
    __shared__ double fin[kRedRows];
    __shared__ double shw[kMainThreads / 32];
    __shared__ int s_task;

    const int tid = threadIdx.x;
    const bool geo = ws.mom[5] != 0.0;
    const double M[5] = {ws.mom[0], ws.mom[1], ws.mom[2], ws.mom[3], ws.mom[4]};

    for (;;) {
        if (tid == 0) s_task = atomicAdd(ws.counter, 1);
        __syncthreads();
        const int task = s_task;
        __syncthreads();
        if (task >= ntasks) break;

        int tile, chunk = 0;
        if (SCATTER && geo) { tile = ntile - 1 - task / nchunk; chunk = task % nchunk; }
        else { if (task >= ntile) continue; tile = ntile - 1 - task; }

        const int I = tile * W;
        const int smax = min(I + W - 1, n - 2);     // highest non-clipped slot
        const int d_begin = (SCATTER && geo) ? chunk * kScatterChunk : 0;
        const int d_end = (SCATTER && geo) ? min(n, d_begin + kScatterChunk) : n;
        // skip empty lag chunks (uniform: every thread reads the same entry)
        if (SCATTER && geo && chunk > 0 && (d_begin >= n || ws.Ld[d_begin] > smax)) continue;

        if (tid < W + 2) {
            const int s = I - 1 + tid;
            const bool in = (s >= 0 && s < n);
            xs[tid] = in ? x[s] : 0.0;
            fs[tid] = in ? (K == 2 ? ws.h[s] : N[s]) : 0.0;
        }
        // Per-task exponent shift of the weight numerators: th ~ x_I (r-1) is
        // carried as th 2^St ~ (r-1), so sum rate*th keeps the dynamic range of
        // the reference's w*rate even on grids spanning hundreds of octaves.
        const int St = -ilogb(x[I]);
        const int St20 = St << 20;
        __syncthreads();

        if (geo) {
            double R[W + 1], TH[W + 1];
#pragma unroll
            for (int t = 0; t <= W; ++t) { R[t] = 0.0; TH[t] = 0.0; }
            const int thi = smax - (I - 1);   // slot index t <= thi
            // lags d >= D0 put every pair on its larger member's own slot (lo = k)
            const int D0 = (K == 1) ? n : ws.counter[1];
            int d = d_begin + tid;
            // phase 1, lags with lo > k: rate per pair, R += rate, TH += rate * th
            for (; d < d_end && d < D0; d += kMainThreads) {
                const int L = __ldg(ws.Ld + d);
                if (L > smax) { d = d_end; break; }   // Ld is nondecreasing in d
                const double B = __ldg(ws.Bd + d), S = __ldg(ws.Sd + d);
                const int jb = I - 1 - L;      // j of slot t is jb + t, k = jb + d + t
                const int tlo = max(0, -jb);
#pragma unroll
                for (int t = 0; t <= W; ++t) {
                    if (t >= tlo && t <= thi) {
                        const int j = jb + t, k = j + d;
                        const double Nj = __ldg(N + j), Nk = __ldg(N + k);
                        const double hj = NeedH<K>::j ? __ldg(ws.h + j) : 0.0;
                        const double hk = NeedH<K>::k ? __ldg(ws.h + k) : 0.0;
                        const double rate = rate_geo<K>(B, S, Nj, hj, Nk, hk);
                        // (fl(x_j + x_k) - x_lo) 2^St on the integer pipe, bit-identical
                        // to the reference's two FP64 additions
                        const double th = sum_minus_scaled(__ldg(x + k), __ldg(x + j), xs[t], St);
                        if (t > 0) R[t] += rate;
                        TH[t] = fma(rate, th, TH[t]);
                    }
                }
            }
#pragma unroll
            for (int t = 0; t <= W; ++t) {
                red[t * kMainThreads + tid] = R[t];
                red[(W + 1 + t) * kMainThreads + tid] = TH[t];
                R[t] = 0.0;
                TH[t] = 0.0;
            }
            // phase 2, lags with lo = k: k is the slot itself, so rate = F_slot * q(j)
            // (F = N, or h for Product); sum q and q * th, multiply by F once
            if constexpr (K != 1) {
                for (; d < d_end; d += kMainThreads) {
                    const int L = __ldg(ws.Ld + d);
                    if (L > smax) break;
                    const double B = __ldg(ws.Bd + d), S = __ldg(ws.Sd + d);
                    const int jb = I - 1 - L;
                    const int tlo = max(0, -jb);
#pragma unroll
                    for (int t = 0; t <= W; ++t) {
                        if (t >= tlo && t <= thi) {
                            const int j = jb + t;
                            const double Nj = __ldg(N + j);
                            const double hj = NeedH<K>::j ? __ldg(ws.h + j) : 0.0;
                            const double q = q_slot<K>(B, S, Nj, hj);
                            const double th = sum_minus_scaled(xs[t], __ldg(x + j), xs[t], St);
                            if (t > 0) R[t] += q;
                            TH[t] = fma(q, th, TH[t]);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t <= W; ++t) {
                    double* r0 = red + t * kMainThreads + tid;
                    double* r1 = red + (W + 1 + t) * kMainThreads + tid;
                    *r0 = fma(fs[t], R[t], *r0);
                    *r1 = fma(fs[t], TH[t], *r1);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < kRedRows; ++r) red[r * kMainThreads + tid] = 0.0;
            const int s_first = max(I - 1, 0);
            if (smax >= s_first) {
                const int t_first = s_first - (I - 1);
                const int t_last = smax - (I - 1);
                const long long blo = dbits(xs[t_first]);
                const long long bhi = dbits(xs[t_last + 1]);
                const double* __restrict__ xsc = x;
                const double xlast = xsc[n - 1];
                for (int j = tid; j <= smax; j += kMainThreads) {
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
                    const double Nj = N[j], hj = ws.h[j], aj = ws.a[j], iaj = ws.ia[j];
                    int t = t_first;
                    double Rc = 0.0, THc = 0.0;
                    for (int k = ka; k < kb; ++k) {
                        const double v = xj + xsc[k];
                        const long long vb = dbits(v);
                        while (t < t_last && dbits(xs[t + 1]) <= vb) {
                            red[t * kMainThreads + tid] += Rc;
                            red[(W + 1 + t) * kMainThreads + tid] += THc;
                            Rc = 0.0; THc = 0.0; ++t;
                        }
                        const double rate = rate_gen<K>(j == k, b0, bbr, bsh, Nj, hj, aj, iaj,
                                                        N[k], ws.h[k], ws.a[k], ws.ia[k]);
                        Rc += rate;
                        THc = fma(rate, scale_pow2(v - xs[t], St20), THc);
                    }
                    red[t * kMainThreads + tid] += Rc;
                    red[(W + 1 + t) * kMainThreads + tid] += THc;
                }
            }
        }
        __syncthreads();

        // fixed-order reduction: 4 chunks of 64 columns per row, then the chunks
        if (tid < kRedRows * 4) {
            const int r = tid >> 2, c = tid & 3;
            const double* p = red + r * kMainThreads + c * 64;
            double s = 0.0;
#pragma unroll 8
            for (int q = 0; q < 64; ++q) s += p[q];
            part4[c][r] = s;
        }
        __syncthreads();
        if (tid < kRedRows) fin[tid] = (part4[0][tid] + part4[1][tid]) + (part4[2][tid] + part4[3][tid]);

        // clipped pairs of bin n-1 (gather: sum of the clip kernel's partials)
        double clip = 0.0;
        if (!SCATTER && I + W > n - 1) {
            const int nbc = (n + kClipWarps - 1) / kClipWarps;
            double s = 0.0;
            for (int b = tid; b < nbc; b += kMainThreads) s += ws.clip_part[b];
            clip = block_sum(s, shw);
        }
        __syncthreads();

        if (tid < W) {
            const int i = I + tid;
            if (i < n) {
                double birth = 0.0;
                // TH is carried times 2^St: undo it on the (per-bin) inverse widths
                if (i <= n - 2)
                    birth = fma(-fin[W + 1 + tid + 1], scalbn(ws.inv_dx[i], -St), fin[tid + 1]);
                if (i >= 1) birth = fma(fin[W + 1 + tid], scalbn(ws.inv_dx[i - 1], -St), birth);
                const bool first = !(SCATTER && geo) || chunk == 0;
                const double death = first ? N[i] * death_factor<K>(x[i], ws.a[i], ws.ia[i], M, b0, bbr, bsh)
                                           : 0.0;
                if constexpr (SCATTER) {
                    const double val = birth - death;
                    if (val != 0.0) atomicAdd(rhs + i, val);
                } else {
                    if (i == n - 1) birth += clip;
                    rhs[i] = rhs[i] + (birth - death);
                }
            }
        }
        __syncthreads();
    }
}

template <int K, bool SC>
cudaError_t launch_k(const AggArgs& a, const AggWs& ws, int num_sms, cudaStream_t s)
{
    const int n = a.n;
    const int nb = agg_prep_blocks(n);
    const int nbc = agg_clip_blocks(n);
    const int ntile = (n + W - 1) / W;
    const int nchunk = SC ? (n + kScatterChunk - 1) / kScatterChunk : 1;
    const long long ntasks_ll = static_cast<long long>(ntile) * nchunk;
    if (ntasks_ll > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int ntasks = static_cast<int>(ntasks_ll);
    const int grid = static_cast<int>(ntasks < 2LL * num_sms ? ntasks : 2LL * num_sms);
    const size_t smem = sizeof(double) * kRedRows * kMainThreads;
    cudaError_t e = cudaFuncSetAttribute(agg_main_kernel<K, SC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    agg_prep_kernel<K><<<nb, kPrepThreads, 0, s>>>(a.N, a.x, n, ws, a.beta0, a.beta_br, a.beta_sh);
    agg_fin_kernel<<<1, 256, 0, s>>>(a.x, n, ws);
    agg_clip_kernel<K, SC><<<nbc, kClipWarps * 32, 0, s>>>(a.N, a.x, a.rhs, n, ws, a.beta0,
                                                          a.beta_br, a.beta_sh);
    const bool prof = g_prof_start && g_prof_stop;
    if (prof) cudaEventRecord(g_prof_start, s);
    agg_main_kernel<K, SC><<<grid, kMainThreads, smem, s>>>(a.N, a.x, a.rhs, ws, n, ntile, nchunk,
                                                            ntasks, a.beta0, a.beta_br, a.beta_sh);
    if (prof) cudaEventRecord(g_prof_stop, s);
    return cudaGetLastError();
}

template <bool SC>
cudaError_t dispatch(const AggArgs& a, const AggWs& ws, int num_sms, cudaStream_t s)
{
    switch (a.kernel) {
    case 0: return launch_k<0, SC>(a, ws, num_sms, s);
    case 1: return launch_k<1, SC>(a, ws, num_sms, s);
    case 2: return launch_k<2, SC>(a, ws, num_sms, s);
    case 3: return launch_k<3, SC>(a, ws, num_sms, s);
    case 4: return launch_k<4, SC>(a, ws, num_sms, s);
    case 5: return launch_k<5, SC>(a, ws, num_sms, s);
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
    return scatter ? dispatch<true>(a, ws, num_sms, s) : dispatch<false>(a, ws, num_sms, s);
}

} // namespace pbe_gb300
