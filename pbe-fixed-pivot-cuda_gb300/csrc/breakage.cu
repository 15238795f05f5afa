// =============================================================================
// breakage.cu -- fixed-pivot breakage RHS for GB300 (sm_103a), FP64.
//
// Reference semantics (acuoci/pbe-fixed-pivot-cuda src/breakage_kernels.cuh):
//   death (:115-133): rhs[j] -= S(x_j) N_j       if S != 0 && N_j > 2.2e-308
//   birth (:160-251): for every parent j and quadrature point q with the same
//     guard, contrib = S_j N_j bw_q, v = x_j t_q; v <= x[0] -> bin 0,
//     v >= x[n-1] -> bin n-1, else split onto lo, lo+1 with
//     eta = (v - x_lo)/(x_{lo+1} - x_lo) (lo from a binary search, :95-105).
//   selection S (:51-65): S0 | S0 v/v_ref | S0 (v/v_ref)^alpha | (v > v_min) S0.
//
// GATHER (deterministic): one thread per fragment (q, j) computes its bracket
// and its two shares; since v = x_j t_q grows with j, the fragments of one q
// landing on bracket m form a contiguous run of j, whose first index is
// recorded in first[q][m]. The gather kernel then gives each output bin i a
// segment of lanes, one per quadrature point, which add in a fixed order the
// hi-shares of bracket i-1 and the lo-shares of bracket i (bin 0 also takes
// the fragments clipped below x[0]), then the death term -S_i N_i.
// SCATTER: one thread per fragment adds its shares with FP64 atomicAdd.
// =============================================================================
#include <cstdlib>
#include <cstring>

#include "pbe_internal.cuh"

namespace pbe_gb300 {
namespace {

// Shares of one fragment: (to lo, to lo+1). Clipped fragments put everything
// into the first share.
__device__ __forceinline__ void frag_shares(const double* __restrict__ x, int n, int lo, double v,
                                            double contrib, double& clo, double& chi)
{
    if (lo < 0 || lo >= n - 1) { clo = contrib; chi = 0.0; return; }
    const double xl = __ldg(x + lo), xh = __ldg(x + lo + 1);
    const double q = contrib / (xh - xl);
    clo = q * (xh - v);
    chi = q * (v - xl);
}

// prep modes: kBrkFull computes everything per call; kBrkTables only the
// grid-only tables (fragment brackets lo, run starts, S per bin) into the
// workspace; kBrkStage the N-dependent shares from those tables, with the
// arithmetic of kBrkFull (bitwise the same shares and sums).
enum { kBrkFull = 0, kBrkTables = 1, kBrkStage = 2 };

template <int F, int MODE>
__global__ void __launch_bounds__(256)
brk_prep_kernel(const double* __restrict__ N, const double* __restrict__ x,
                const double* __restrict__ t_q, const double* __restrict__ bw_q, int n, int nq,
                BrkWs ws, double S0, double v_ref, double alpha, double v_min)
{
    __shared__ double sh[8];
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool live = idx < static_cast<long long>(n) * nq;   // every lane takes part in the shuffle
    const int lane = threadIdx.x & 31;
    int q = 0, j = 0, lo = -2;
    double clipped = 0.0;
    double tq = 0.0;
    if (live) {
        q = static_cast<int>(idx / n);
        j = static_cast<int>(idx - static_cast<long long>(q) * n);
        const double xj = x[j];
        tq = t_q[q];
        const double v = xj * tq;
        double S;
        if constexpr (MODE == kBrkStage) {
            S = ws.Ssel[j];
            lo = ws.lo[idx];
        } else {
            S = selection<F>(xj, S0, v_ref, alpha, v_min);
            lo = frag_bracket(x, n, v);
        }
        if constexpr (MODE == kBrkTables) {
            ws.lo[idx] = lo;
            if (q == 0) ws.Ssel[j] = S;
        } else {
            const double Nj = N[j];
            const bool active = (S != 0.0) && (Nj > kBreakageNMin);
            const double contrib = active ? S * Nj * bw_q[q] : 0.0;
            double clo, chi;
            frag_shares(x, n, lo, v, contrib, clo, chi);
            ws.clo[idx] = clo;
            ws.chi[idx] = chi;
            if (lo < 0) clipped = clo;           // all of it goes to bin 0
            if (q == 0) ws.SN[j] = active ? S * Nj : 0.0;
        }
    }
    if constexpr (MODE != kBrkStage) {
        // bracket of the previous parent's fragment (same q): the lane below has it
        const int lo_left = __shfl_up_sync(0xffffffffu, lo, 1);
        if (live) {
            // run starts: first[q][m+1] = j for every bracket m in (lo(j-1), lo(j)]
            int* fq = ws.first + static_cast<long long>(q) * (n + 2);
            const int lo_prev = (j == 0) ? -2
                              : (lane > 0 ? lo_left : frag_bracket_below(x, n, x[j - 1] * tq, lo));
            for (int m = max(lo_prev + 1, -1); m <= lo; ++m) fq[m + 1] = j;
            if (j == n - 1)
                for (int m = max(lo + 1, -1); m <= n; ++m) fq[m + 1] = n;
        }
    }
    if constexpr (MODE != kBrkTables) {
        // this block's fragments clipped below x[0], summed in a fixed order (most
        // blocks have none: one barrier tells)
        if (__syncthreads_or(clipped != 0.0)) {
            const double cs = block_sum(clipped, sh);
            if (threadIdx.x == 0) ws.clipsum[blockIdx.x] = cs;
        } else if (threadIdx.x == 0) {
            ws.clipsum[blockIdx.x] = 0.0;
        }
    }
}

// Output bins in groups of 32/nqp per warp, nqp = n_quad rounded up to a power
// of two (<= 32): lane l works on bin base + l / nqp and quadrature points
// q = l % nqp (+ nqp, ...), walking that q's few fragments of brackets i-1 and
// i; a fixed butterfly over the nqp lanes sums them. Bin 0 also collects every
// fragment clipped below x[0] (thousands on fine grids), pre-summed per prep
// block.
__global__ void __launch_bounds__(256)
brk_gather_kernel(double* __restrict__ rhs, int n, int nq, BrkWs ws)
{
    __shared__ double sh[8];
    int nqp = 1;
    while (nqp < nq && nqp < 32) nqp <<= 1;
    const int per_warp = 32 / nqp;
    const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int base = warp * per_warp;
    // fragments clipped below x[0] (all deposited on bin 0): block 0 adds the
    // prep blocks' sums in a fixed order
    double clipped = 0.0;
    if (blockIdx.x == 0) {
        const int nbp = static_cast<int>((static_cast<long long>(n) * nq + 255) / 256);
        double part = 0.0;
        for (int b = threadIdx.x; b < nbp; b += blockDim.x) part += ws.clipsum[b];
        clipped = block_sum(part, sh);
    }
    if (base >= n) return;                   // whole warp
    const int i = base + lane / nqp;
    double acc = 0.0;
    if (i < n) {
        for (int q = lane % nqp; q < nq; q += nqp) {
            const int* fq = ws.first + static_cast<long long>(q) * (n + 2);
            const double* clo = ws.clo + static_cast<long long>(q) * n;
            const double* chi = ws.chi + static_cast<long long>(q) * n;
            // clamp: entries are in [0, n] for monotone brackets (t_q > 0)
            const int fa = min(max(fq[i], 0), n);         // first j with lo >= i-1
            const int fb = min(max(fq[i + 1], fa), n);    // first j with lo >= i
            const int fc = min(max(fq[i + 2], fb), n);    // first j with lo >= i+1
            if (i > 0) for (int j = fa; j < fb; ++j) acc += chi[j];   // lo == i-1
            // (lo == -1 for i == 0: the clipped fragments, added below)
            for (int j = fb; j < fc; ++j) acc += clo[j];              // lo == i
        }
    }
    for (int o = nqp >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (i < n && (lane % nqp) == 0) {
        if (i == 0) acc += clipped;
        rhs[i] = (rhs[i] - ws.SN[i]) + acc;
    }
}

// ---------------------------------------------------------------------------
// Gather in one pass (the drop-in calls): block b >= 1 = 32 brackets
// c = i0 - 1 + lane, i0 = 1 + 31 (b - 1), x W warps (W = min(n_quad, 4)); warp
// w takes the quadrature points q = w, w + W, ..., and the block writes the 31
// bins i0 .. i0 + 30. A lane walks the parents whose fragment x_j t_q has
// bracket c -- the index range [f(c), f(c + 1)), f(c) the first parent whose
// fragment reaches bracket c (brackets grow with j for t_q > 0), guessed from
// FP32 logs and confirmed by exact tests of the guess and its neighbours; f(c + 1)
// from the next lane -- and forms each fragment's two shares once: the lower
// one for bin c, the upper one for bin c + 1 (4 FP64 instructions per
// fragment and 2 per test). Bin i = i0 + lane adds its own upper shares and
// the next lane's lower shares; bracket n - 1 (fragments at or above x[n-1])
// is all bin n-1's. Block 0 writes bin 0 alone (brk_bin0). Sums run in a
// fixed order (fragments by j, points by q within a warp, warps in order):
// bitwise reproducible.
// ---------------------------------------------------------------------------
constexpr int kBinWarpsMax = 4;
constexpr int kBrkBins = 31;            // bins written per block (32 brackets)

// S_j N_j with the reference's guard (S != 0, N_j > 2.2e-308), from the
// cache `SN` when the selection needs it (Linear, PowerLaw), else inline.
template <int F>
__device__ __forceinline__ double bin_sn(const double* __restrict__ N, const double* __restrict__ x,
                                        const double* __restrict__ SN, int j, double S0,
                                        double v_min)
{
    if constexpr (F == 1 || F == 2) {
        return SN[j];
    } else {
        // comparisons on bit patterns (the integer pipe): x_j > 0, so
        // x_j > v_min <=> bits(x_j) > bits(v_min) for any v_min, and
        // N_j > 2.2e-308 <=> bits(N_j) > bits(2.2e-308) for any N_j
        const double S = (F == 0) ? S0 : ((dbits(__ldg(x + j)) > dbits(v_min)) ? S0 : 0.0);
        const double Nj = __ldg(N + j);
        return (S != 0.0 && dbits(Nj) > dbits(kBreakageNMin)) ? S * Nj : 0.0;
    }
}

// The parent's factor of its fragments' shares: N_j (guarded: 0 where the
// reference skips the parent) for Constant / Threshold, whose S0 goes into
// the per-lane factor; S_j N_j from the cache otherwise.
template <int F>
__device__ __forceinline__ double bin_unit(const double* __restrict__ N, const double* __restrict__ x,
                                          const double* __restrict__ SN, int j, double v_min)
{
    if constexpr (F == 1 || F == 2) {
        return SN[j];
    } else {
        const bool on = (F == 0) || dbits(__ldg(x + j)) > dbits(v_min);
        const double Nj = __ldg(N + j);
        return (on && dbits(Nj) > dbits(kBreakageNMin)) ? Nj : 0.0;
    }
}

// First parent j in [0, n] whose fragment x_j t_q has bracket >= ib
// (ib = 0: x_j t_q > x[0]; 1 <= ib <= n - 1: x_j t_q >= x[ib]; ib >= n: n),
// given a lower bound lb <= the answer and a guess: the exact test
// fl(x_j t_q) on the guess, a gallop away from it until the answer is
// bracketed, then bisection. One or two tests when the guess is right (on a
// geometric grid the first parents of consecutive bins are consecutive).
__device__ __forceinline__ int first_parent_near(const double* __restrict__ x, int n, int ib,
                                                 double tq, int lb, int guess)
{
    if (ib >= n) return n;
    const long long xb = dbits(__ldg(x + ib));
    auto P = [&](int j) {                     // bracket of fragment j >= ib; P(n) := true
        if (j >= n) return true;
        const long long vb = dbits(__ldg(x + j) * tq);
        return ib == 0 ? (vb > xb && vb > 0) : vb >= xb;
    };
    int g = guess < lb ? lb : (guess > n ? n : guess);
    int a, b;                                 // answer in (a, b]: P(b), a < lb or !P(a)
    if (P(g)) {
        b = g;
        int step = 1;
        a = g - 1;
        while (a >= lb && P(a)) {
            b = a;
            step <<= 1;
            a = b - step;
        }
        if (a < lb - 1) a = lb - 1;
    } else {
        a = g;
        int step = 1;
        b = g + 1 < n ? g + 1 : n;
        while (!P(b)) {
            a = b;
            step <<= 1;
            b = a + step < n ? a + step : n;
        }
    }
    while (b - a > 1) {
        const int mid = (a + b) >> 1;
        if (P(mid)) b = mid; else a = mid;
    }
    return b;
}

// first_parent of bin ib from a guess, testing the guess and both neighbours
// at once (three independent loads and products): the answer when it is one
// of them -- on a geometric grid it is -- else the gallop of
// first_parent_near. Also returns the fragment volumes fl(x_f t_q) of the
// answer f and, when it was formed, of f + 1.
struct FirstParent {
    int f;
    bool has_v1;
    double v, v1;
};
__device__ __forceinline__ FirstParent first_parent_spec(const double* __restrict__ x, int n, int ib,
                                                         double tq, int guess)
{
    FirstParent r{n, false, 0.0, 0.0};
    if (ib >= n) return r;
    const long long xb = dbits(__ldg(x + ib));
    auto P = [&](double v) {                   // bracket of a fragment volume >= ib
        const long long vb = dbits(v);
        return ib == 0 ? (vb > xb && vb > 0) : vb >= xb;
    };
    const int g = guess < 0 ? 0 : (guess > n - 1 ? n - 1 : guess);
    const double vm = __ldg(x + (g >= 1 ? g - 1 : 0)) * tq;
    const double v0 = __ldg(x + g) * tq;
    const double vp = __ldg(x + (g + 1 < n ? g + 1 : g)) * tq;
    const bool pm = g >= 1 && P(vm);
    const bool p0 = P(v0);
    const bool pp = g + 1 >= n || P(vp);       // P(n) := true
    if (!pm && p0) {
        r.f = g; r.v = v0; r.v1 = vp; r.has_v1 = g + 1 < n;
    } else if (!p0 && pp) {
        r.f = g + 1; r.v = vp;                 // f = n when no parent reaches ib
    } else {
        r.f = first_parent_near(x, n, ib, tq, 0, g);
        if (r.f < n) r.v = __ldg(x + r.f) * tq;
    }
    return r;
}

// Index guess of the first parent of bin ib for the point with log2(t_q) = ltq
// (geometric grid through x[0] and x[n-1]), from lxb = log2_approx(x[ib]).
__device__ __forceinline__ int first_parent_guess(float lxb, float ltq, float lx0, float inv_span, int n)
{
    float gf = (lxb - ltq - lx0) * inv_span;
    gf = fminf(fmaxf(gf, 0.0f), static_cast<float>(n));
    return static_cast<int>(gf);
}

// One (bracket, point): the parents [f0, f1), v0 the fragment volume of parent
// f0. Adds sum u_j bw to A (the whole contribution) and, for c in [0, n-2],
// sum u_j bw (v - x_c) to H (the upper share before the factor 1/dx_c); the
// lower share is A - H/dx_c. c = n - 1: all of it is bin n-1's (H stays 0).
template <int F>
__device__ __forceinline__ void bracket_shares(const double* __restrict__ N, const double* __restrict__ x,
                                               const double* __restrict__ SN, double v_min, int f0,
                                               int f1, double v0, double tq, double bw, double xc,
                                               bool mid, bool top, double& A, double& H)
{
    if (f0 >= f1) return;
    if (mid) {
        const double a0 = bin_unit<F>(N, x, SN, f0, v_min) * bw;
        H = fma(a0, v0 - xc, H);
        A += a0;
        for (int j = f0 + 1; j < f1; ++j) {
            const double a = bin_unit<F>(N, x, SN, j, v_min) * bw;
            H = fma(a, __ldg(x + j) * tq - xc, H);
            A += a;
        }
    } else if (top) {
        for (int j = f0; j < f1; ++j) A = fma(bin_unit<F>(N, x, SN, j, v_min), bw, A);
    }
}

// Block 0: bin 0 alone -- the fragments at or below x[0] (bracket -1, all of
// them bin 0's) and the lower shares of bracket 0 (or, when n = 1, all of
// bracket 0). Thread q takes point q (q = tid, tid + T, ...): f_q(0), f_q(1)
// and bracket 0's fragments; the fragments of bracket -1 are the parents
// j < f_q(0), summed as bw_q U(f_q(0)) with U(f) = sum_{j < f} u_j from one
// block-wide prefix of u over [0, max_q f_q(0)) (contiguous chunks per
// thread, a warp scan by a fixed shuffle pattern, warp totals in order). A
// warp walking those parents point by point was the kernel's long pole
// (~4000 parents per point on a 512-bins-per-doubling grid).
template <int F>
__device__ __forceinline__ void brk_bin0(const double* __restrict__ N, const double* __restrict__ x,
                                         const double* __restrict__ t_q, const double* __restrict__ bw_q,
                                         double* __restrict__ rhs, int n, int nq,
                                         const double* __restrict__ SN, double S0, double v_min,
                                         float lx0, float inv_span)
{
    __shared__ int s_fmax[kBinWarpsMax];
    __shared__ double s_wtot[kBinWarpsMax];
    __shared__ double s_pre[32 * kBinWarpsMax];
    constexpr bool kS0 = (F == 0 || F == 3);
    const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, w = tid >> 5, W = T >> 5;
    const bool mid0 = n >= 2;                  // bracket 0 is [x0, x1); else all of it is bin 0's
    const double x1 = mid0 ? __ldg(x + 1) : 0.0;
    const double inv0 = mid0 ? 1.0 / (x1 - __ldg(x)) : 0.0;
    const float lx1 = mid0 ? log2_approx(x1) : 0.0f;
    auto f0_of = [&](double tq, float ltq) {
        return first_parent_spec(x, n, 0, tq, first_parent_guess(lx0, ltq, lx0, inv_span, n)).f;
    };
    int fm = 0;
    double term = 0.0;
    for (int q = tid; q < nq; q += T) {
        const double tq = __ldg(t_q + q), bw = __ldg(bw_q + q);
        const float ltq = __log2f(static_cast<float>(tq));
        const int f0 = f0_of(tq, ltq);
        const int f1 = mid0 ? first_parent_spec(x, n, 1, tq, first_parent_guess(lx1, ltq, lx0, inv_span, n)).f
                            : n;
        fm = max(fm, f0);
        double lo = 0.0;
        for (int j = f0; j < f1; ++j) {
            const double u = bin_unit<F>(N, x, SN, j, v_min);
            lo = mid0 ? fma(u, (x1 - __ldg(x + j) * tq) * inv0, lo) : lo + u;
        }
        term = fma(bw, lo, term);
    }
    for (int o = 16; o > 0; o >>= 1) fm = max(fm, __shfl_xor_sync(0xffffffffu, fm, o));
    if (lane == 0) s_fmax[w] = fm;
    __syncthreads();
    int fmax = 0;
    for (int k = 0; k < W; ++k) fmax = max(fmax, s_fmax[k]);
    const int chunk = (fmax + T - 1) / T;
    const int j0 = min(fmax, tid * chunk), j1 = min(fmax, j0 + chunk);
    double cs = 0.0;
    for (int j = j0; j < j1; ++j) cs += bin_unit<F>(N, x, SN, j, v_min);
    double sc = cs;                                            // inclusive scan in the warp
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, sc, o);
        if (lane >= o) sc += t;
    }
    double ex = __shfl_up_sync(0xffffffffu, sc, 1);            // exclusive
    if (lane == 0) ex = 0.0;
    if (lane == 31) s_wtot[w] = sc;
    __syncthreads();
    double wbase = 0.0;
    for (int k = 0; k < w; ++k) wbase += s_wtot[k];
    s_pre[tid] = wbase + ex;                                   // sum of u_j, j < tid * chunk
    __syncthreads();
    if (chunk > 0) {
        for (int q = tid; q < nq; q += T) {
            const double tq = __ldg(t_q + q);
            const int f = f0_of(tq, __log2f(static_cast<float>(tq)));
            const int t = min(f / chunk, T - 1);
            double pre = s_pre[t];
            for (int j = t * chunk; j < f; ++j) pre += bin_unit<F>(N, x, SN, j, v_min);
            term = fma(__ldg(bw_q + q), pre, term);
        }
    }
    const double total = block_sum(term, s_wtot) * (kS0 ? S0 : 1.0);
    if (tid == 0) {
        double sn0;
        if constexpr (F == 1 || F == 2) sn0 = SN[0];
        else sn0 = bin_sn<F>(N, x, SN, 0, S0, v_min);
        rhs[0] = (rhs[0] - sn0) + total;
    }
}

template <int F>
__global__ void __launch_bounds__(32 * kBinWarpsMax)
brk_bin_kernel(const double* __restrict__ N, const double* __restrict__ x,
               const double* __restrict__ t_q, const double* __restrict__ bw_q,
               double* __restrict__ rhs, int n, int nq, const double* __restrict__ SN,
               double S0, double v_ref, double alpha, double v_min)
{
    if ((F == 0 || F == 3) && S0 == 0.0) return;     // S = 0 everywhere: no breakage at all
    __shared__ double s_acc[kBinWarpsMax][32];
    // index of a volume on the geometric grid through x[0] and x[n-1] (guesses only)
    const float lx0 = log2_approx(__ldg(x));
    const float span = log2_approx(__ldg(x + n - 1)) - lx0;
    const float inv_span = (n > 1 && span > 0.0f) ? static_cast<float>(n - 1) / span : 0.0f;
    if (blockIdx.x == 0) {
        brk_bin0<F>(N, x, t_q, bw_q, rhs, n, nq, SN, S0, v_min, lx0, inv_span);
        return;
    }
    const int i0 = 1 + (blockIdx.x - 1) * kBrkBins;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;

    const int c = i0 - 1 + lane;               // this lane's bracket (>= 0)
    const bool mid = c <= n - 2;               // x[c] <= v < x[c+1]
    const bool top = c == n - 1;               // v >= x[n-1]: all to bin n-1
    const int ib = c < n ? c : n - 1;
    const double xc = __ldg(x + ib);
    const double xc1 = mid ? __ldg(x + c + 1) : 0.0;
    const double inv = mid ? 1.0 / (xc1 - xc) : 0.0;
    const float lxc = log2_approx(xc);
    // lane 31 also needs f(i0 + 31)
    const int ibt = min(i0 + 31, n - 1);
    const float lxt = log2_approx(__ldg(x + ibt));
    // selections with a per-bin S of S0 or 0 (Constant, Threshold): the parent
    // adds N_j, S0 multiplies the lane's sums once at the end, as 1/dx_c does
    constexpr bool kS0 = (F == 0 || F == 3);
    double A = 0.0, H = 0.0;                   // this warp's points, in q order
    const int cb = c;
    const long long xb = dbits(xc);            // threshold of bracket c (c < n)
    for (int q = w; q < nq; q += W) {
        const double tq = __ldg(t_q + q), bw = __ldg(bw_q + q);
        const float ltq = __log2f(static_cast<float>(tq));
        // f(c) from a guess g: the tests of g - 1, g, g + 1 need three fragment
        // volumes; on a geometric grid the neighbour lanes' guesses are g - 1
        // and g + 1, so one product per lane plus one more (the ends of the
        // warp, misaligned guesses) covers them
        int g = first_parent_guess(lxc, ltq, lx0, inv_span, n);
        g = g > n - 1 ? n - 1 : g;
        const double v0 = __ldg(x + g) * tq;
        const int gl = __shfl_up_sync(0xffffffffu, g, 1);
        const double vl = __shfl_up_sync(0xffffffffu, v0, 1);
        const int gr = __shfl_down_sync(0xffffffffu, g, 1);
        const double vr = __shfl_down_sync(0xffffffffu, v0, 1);
        const bool have_m = lane > 0 && gl == g - 1;
        const bool have_p = lane < 31 && gr == g + 1;
        const int e = !have_m ? g - 1 : g + 1;
        const double ve = __ldg(x + min(max(e, 0), n - 1)) * tq;
        double vm = have_m ? vl : ve;
        double vp = have_p ? vr : ve;
        if (!have_m && !have_p && g + 1 < n) vp = __ldg(x + g + 1) * tq;   // rare
        int f = n;
        bool has_v1 = false;
        double v = 0.0, v1 = 0.0;
        if (c < n) {
            auto P = [&](double vv) {            // fragment bracket >= cb
                const long long vb = dbits(vv);
                return cb == 0 ? (vb > xb && vb > 0) : vb >= xb;
            };
            const bool pm = g >= 1 && P(vm);
            const bool p0 = P(v0);
            const bool pp = g + 1 >= n || P(vp);  // P(n) := true
            if (!pm && p0) {
                f = g; v = v0; v1 = vp; has_v1 = g + 1 < n;
            } else if (!p0 && pp) {
                f = g + 1; v = vp;
            } else {
                f = first_parent_near(x, n, cb, tq, 0, g);
                if (f < n) v = __ldg(x + f) * tq;
            }
        }
        // lane 31 also needs f(c + 1): from its own volumes when they decide it
        int ft = n;
        if (lane == 31 && c + 1 < n && f < n) {
            const long long xb1 = dbits(__ldg(x + c + 1));
            if (dbits(v) >= xb1) ft = f;
            else if (has_v1 && dbits(v1) >= xb1) ft = f + 1;
            else ft = first_parent_near(x, n, c + 1, tq, f, f + 2);
        }
        // every lane runs every shuffle (full mask), then selects
        const int up = __shfl_down_sync(0xffffffffu, f, 1);
        const int fn = (lane < 31) ? up : ft;                   // f(c + 1)
        bracket_shares<F>(N, x, SN, v_min, f, fn, v, tq, bw, xc, mid, top, A, H);
    }
    // bin c: the lower shares A - H/dx_c; bin c + 1: the upper shares H/dx_c
    const double s0 = kS0 ? S0 : 1.0;
    const double hi = mid ? H * inv * s0 : 0.0;
    const double lo = A * s0 - hi;
    const double lo_next = __shfl_down_sync(0xffffffffu, lo, 1);
    const double acc = hi + lo_next;                           // bin i0 + lane (lane < 31)
    s_acc[w][lane] = acc;
    __syncthreads();
    const int i = i0 + lane;
    if (w == 0 && lane < kBrkBins && i < n) {
        double t = 0.0;
        for (int kq = 0; kq < W; ++kq) t += s_acc[kq][lane];
        double sn_i;
        if constexpr (F == 1 || F == 2) sn_i = SN[i];
        else sn_i = bin_sn<F>(N, x, SN, i, S0, v_min);
        rhs[i] = (rhs[i] - sn_i) + t;
    }
}

// S_j N_j with the reference's guard, one thread per bin (Linear and
// PowerLaw selections: one division or pow per bin instead of per fragment).
template <int F>
__global__ void __launch_bounds__(256)
brk_sn_kernel(const double* __restrict__ N, const double* __restrict__ x, int n, double* SN,
              double S0, double v_ref, double alpha, double v_min)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double S = selection<F>(x[j], S0, v_ref, alpha, v_min);
    const double Nj = N[j];
    SN[j] = (S != 0.0 && Nj > kBreakageNMin) ? S * Nj : 0.0;
}

int brk_gather_path()
{
    // PBE_GB300_BRK_PATH=prep: the per-fragment prep + gather kernels instead
    static const int path = []() {
        const char* e = std::getenv("PBE_GB300_BRK_PATH");
        return (e && std::strcmp(e, "prep") == 0) ? 1 : 0;
    }();
    return path;
}

template <int F>
__global__ void __launch_bounds__(256)
brk_scatter_kernel(const double* __restrict__ N, const double* __restrict__ x,
                   const double* __restrict__ t_q, const double* __restrict__ bw_q, double* rhs,
                   int n, int nq, double S0, double v_ref, double alpha, double v_min)
{
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(n) * nq) return;
    const int q = static_cast<int>(idx / n);
    const int j = static_cast<int>(idx - static_cast<long long>(q) * n);
    const double xj = x[j], Nj = N[j];
    const double S = selection<F>(xj, S0, v_ref, alpha, v_min);
    if (!((S != 0.0) && (Nj > kBreakageNMin))) return;
    if (q == 0) atomicAdd(rhs + j, -(S * Nj));
    const double contrib = S * Nj * bw_q[q];
    const double v = xj * t_q[q];
    const int lo = frag_bracket(x, n, v);
    double clo, chi;
    frag_shares(x, n, lo, v, contrib, clo, chi);
    if (lo < 0) { atomicAdd(rhs, clo); return; }
    atomicAdd(rhs + lo, clo);
    if (lo < n - 1) atomicAdd(rhs + lo + 1, chi);
}

template <int F>
cudaError_t launch_f(const BrkArgs& a, bool scatter, void* ws_base, cudaStream_t s, int kind)
{
    const long long m = static_cast<long long>(a.n) * a.n_quad;
    const int grid = static_cast<int>((m + 255) / 256);
    if (scatter) {
        brk_scatter_kernel<F><<<grid, 256, 0, s>>>(a.N, a.x, a.t_q, a.bw_q, a.rhs, a.n, a.n_quad,
                                                   a.S0, a.v_ref, a.alpha, a.v_min);
    } else {
        BrkWs ws;
        brk_ws_layout(a.n, a.n_quad, static_cast<char*>(ws_base), &ws);
        if (kind == kBrkFull && brk_gather_path() == 0) {
            if (F == 1 || F == 2)
                brk_sn_kernel<F><<<(a.n + 255) / 256, 256, 0, s>>>(a.N, a.x, a.n, ws.SN, a.S0,
                                                                  a.v_ref, a.alpha, a.v_min);
            const int W = a.n_quad < kBinWarpsMax ? a.n_quad : kBinWarpsMax;
            brk_bin_kernel<F><<<1 + (a.n - 1 + kBrkBins - 1) / kBrkBins, 32 * W, 0, s>>>(
                a.N, a.x, a.t_q, a.bw_q, a.rhs, a.n, a.n_quad, ws.SN, a.S0, a.v_ref, a.alpha,
                a.v_min);
            return cudaGetLastError();
        }
        if (kind == kBrkTables) {
            brk_prep_kernel<F, kBrkTables><<<grid, 256, 0, s>>>(a.N, a.x, a.t_q, a.bw_q, a.n,
                                                                a.n_quad, ws, a.S0, a.v_ref,
                                                                a.alpha, a.v_min);
            return cudaGetLastError();
        }
        if (kind == kBrkStage)
            brk_prep_kernel<F, kBrkStage><<<grid, 256, 0, s>>>(a.N, a.x, a.t_q, a.bw_q, a.n,
                                                               a.n_quad, ws, a.S0, a.v_ref,
                                                               a.alpha, a.v_min);
        else
            brk_prep_kernel<F, kBrkFull><<<grid, 256, 0, s>>>(a.N, a.x, a.t_q, a.bw_q, a.n,
                                                              a.n_quad, ws, a.S0, a.v_ref,
                                                              a.alpha, a.v_min);
        int nqp = 1;
        while (nqp < a.n_quad && nqp < 32) nqp <<= 1;
        const int per_block = 8 * (32 / nqp);               // bins per 256-thread block
        brk_gather_kernel<<<(a.n + per_block - 1) / per_block, 256, 0, s>>>(a.rhs, a.n, a.n_quad, ws);
    }
    return cudaGetLastError();
}

} // namespace

namespace {
cudaError_t brk_dispatch(const BrkArgs& a, bool scatter, void* ws_base, cudaStream_t s, int kind)
{
    switch (a.selection) {
    case 0: return launch_f<0>(a, scatter, ws_base, s, kind);
    case 1: return launch_f<1>(a, scatter, ws_base, s, kind);
    case 2: return launch_f<2>(a, scatter, ws_base, s, kind);
    case 3: return launch_f<3>(a, scatter, ws_base, s, kind);
    default: return cudaErrorInvalidValue;
    }
}
} // namespace

cudaError_t brk_launch(const BrkArgs& a, bool scatter, void* ws_base, cudaStream_t s)
{
    return brk_dispatch(a, scatter, ws_base, s, kBrkFull);
}

cudaError_t brk_tables_launch(const BrkArgs& a, void* ws_base, cudaStream_t s)
{
    return brk_dispatch(a, false, ws_base, s, kBrkTables);
}

cudaError_t brk_stage_launch(const BrkArgs& a, void* ws_base, cudaStream_t s)
{
    return brk_dispatch(a, false, ws_base, s, kBrkStage);
}

} // namespace pbe_gb300
