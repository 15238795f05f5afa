// =============================================================================
// vjp_tile.cuh -- the aggregation VJP row-tile task, shared by the
// single-instance kernel (vjp.cu) and the batched-cell kernel (batch_vjp.cu).
//
// A task owns the VW = kTileW rows [I, I + VW) of one cell and accumulates,
// per row m, up to two partner sums of P (the lambda interpolated at the
// pair's birth volume) times N_k (or x_k N_k) times the lag factor (see
// vjp.cu for the derivation). It runs on a group of T threads (runtime
// value, named barrier, like agg_tile.cuh); the T partials of every row are
// reduced in a fixed order.
// =============================================================================
#pragma once

#include "agg_tile.cuh"

namespace pbe_gb300 {

constexpr int kVW = kTileW;              // rows per task
constexpr int kVRows = 2 * kVW;          // two accumulators per row

// sum_k f(m,k) N_k (or lambda_k N_k) from the moments mo[0..4].
template <int K, int X>   // X: 0 = beta0 / Brownian part, 1 = shear part
__device__ __forceinline__ double moment_factor(double xm, double am, double iam, const double* mo)
{
    if constexpr (K == 0) return mo[1];
    else if constexpr (K == 1) return fma(xm, mo[1], mo[4]);
    else if constexpr (K == 2) return xm * mo[4];
    else if constexpr (X == 0) return fma(am, mo[0], iam * mo[2]) + 2.0 * mo[1];
    else return fma(xm, mo[1], (3.0 * am) * fma(am, mo[2], mo[3])) + mo[4];
}

// One cell as seen by a VJP row task.
struct VjpCellView {
    const double* x;       // pivots [n]
    const double* N;       // [n]
    const double* h;       // x N [n]
    const double* lam;     // lambda = dL/drhs [n]
    const double* D;       // (lambda_{i+1} - lambda_i) / (x_{i+1} - x_i) [n]
    const double* a;       // x^(1/3)
    const double* ia;      // x^(-1/3)
    const double* Bf;      // Brownian lag factor (rho + 1/rho + 2) ...
    const double* Sf;      // shear lag factor (1 + rho)^3 ...
    const double* Sl;      // ... the same times x_0 / x_d (lower partners: f = x_m Sl)
    const int*    Ld;      // bracket offset of lag d
    double lag0_scale;     // ... times lag0_scale at d = 0 (tables that carry the pair 1/2 use 2)
    int n;
    bool geo;
};

constexpr int kVMaxGroups = kMainThreads / 32;

struct VjpShared {
    double part[kVMaxGroups][kVRows];     // 32-column chunk partials (chunk g*T/32 + c)
    double fin[kVMaxGroups][kVRows];      // R0[0..VW), R1[0..VW) of the task
    double gsh[kVMaxGroups][kVW][2];      // per-row parameter partials
    double cinfo[kVMaxGroups][16];        // per-task cell values (batched)
};

// Rows of a geometric-grid pass: t in [T0, T0 + kVPass) of the task.
#ifndef PBE_VJP_PASS
#define PBE_VJP_PASS 6
#endif
constexpr int kVPass = PBE_VJP_PASS;
static_assert(kVW % kVPass == 0 && kVW / kVPass <= 3, "row passes must split the task's rows in one to three");

template <int K, int T0>
__device__ __forceinline__ void vjp_geo_rows(const VjpCellView& v, int I, int r_begin, int r_end,
                                             int tmax, double lamlast, double* R0, double* R1,
                                             int lane, int T)
{
    const int n = v.n;
    const double* __restrict__ x = v.x;
    const double* __restrict__ N = v.N;
    const double* __restrict__ h = v.h;
    const double* __restrict__ lam = v.lam;
    const double* __restrict__ D = v.D;
    for (int d = r_begin + lane; d < r_end; d += T) {
        const int L = __ldg(v.Ld + d);
        const double sc = (d == 0) ? v.lag0_scale : 1.0;
        const double Bf = __ldg(v.Bf + d) * sc, Sf = __ldg(v.Sf + d) * sc;
        // upper visits: partner k = m + d
#pragma unroll
        for (int t = T0; t < T0 + kVPass; ++t) {
            const int m = I + t, k = m + d;
            if (t < tmax && k < n) {
                const double Nk = __ldg(N + k);
                const int lo = (L >= kLagClipAll) ? n : m + L;
                double P;
                if (lo >= n - 1) {
                    P = lamlast;
                } else {
                    const double th = sum_minus_scaled(__ldg(x + k), __ldg(x + m),
                                                       __ldg(x + lo), 0);
                    P = fma(th, __ldg(D + lo), __ldg(lam + lo));
                }
                if constexpr (K == 2) {
                    R0[t] = fma(P, __ldg(h + k), R0[t]);
                } else {
                    const double t1 = P * Nk;
                    if constexpr (K == 0) R0[t] += t1;
                    if constexpr (K == 1) { R0[t] += t1; R1[t] = fma(P, __ldg(h + k), R1[t]); }
                    if constexpr (K == 3 || K == 5) R0[t] = fma(t1, Bf, R0[t]);
                    if constexpr (K == 4 || K == 5) R1[t] = fma(t1, Sf, R1[t]);
                }
            }
        }
    }
    for (int d = r_begin + lane; d < r_end; d += T) {
        // lower visits: partner k = m - d (d >= 1); a lag whose every pair
        // is clipped (L = kLagClipAll) gives lo >= n - 1 -> P = lambda_{n-1}
        if (d == 0) continue;
        const int L = __ldg(v.Ld + d);
        const double Bf = __ldg(v.Bf + d), Sl = __ldg(v.Sl + d);
        const int e = L - d;
#pragma unroll
        for (int t = T0; t < T0 + kVPass; ++t) {
            const int m = I + t, k = m - d;
            if (t < tmax && k >= 0) {
                const int lo = m + e;
                double P;
                if (lo >= n - 1) {
                    P = lamlast;
                } else {
                    const double th = sum_minus_scaled(__ldg(x + m), __ldg(x + k),
                                                       __ldg(x + lo), 0);
                    P = fma(th, __ldg(D + lo), __ldg(lam + lo));
                }
                if constexpr (K == 2) {
                    R0[t] = fma(P, __ldg(h + k), R0[t]);
                } else {
                    const double Nk = __ldg(N + k);
                    if constexpr (K == 0) R0[t] = fma(P, Nk, R0[t]);
                    if constexpr (K == 1) { R0[t] = fma(P, Nk, R0[t]); R1[t] = fma(P, __ldg(h + k), R1[t]); }
                    if constexpr (K >= 3) {
                        const double t1 = P * Nk;
                        if constexpr (K == 3 || K == 5) R0[t] = fma(t1, Bf, R0[t]);
                        if constexpr (K == 4 || K == 5) R1[t] = fma(t1, Sl, R1[t]);
                    }
                }
            }
        }
    }
}

// Row sums of the task's rows into sm.fin[G.g]; red: the group's first column
// of the kVRows x kMainThreads reduction buffer (row stride kMainThreads).
// Row sums over the partner range [r_begin, r_end) (lags on a geometric
// grid, partner indices otherwise); the whole range is [0, n).
template <int K>
__device__ __forceinline__ void vjp_tile_accumulate(const VjpCellView& v, int I, int r_begin,
                                                    int r_end, double* red, VjpShared& sm,
                                                    const TileGroup& G)
{
    constexpr int VW = kVW;
    constexpr int RS = kMainThreads;
    const int n = v.n;
    const int lane = G.lane, T = G.T;
    const int tmax = min(VW, n - I);          // rows I .. I+tmax-1
    const double lamlast = v.lam[n - 1];
    const double* __restrict__ x = v.x;
    const double* __restrict__ N = v.N;
    const double* __restrict__ h = v.h;
    const double* __restrict__ lam = v.lam;
    const double* __restrict__ D = v.D;

    double R0[VW], R1[VW];
#pragma unroll
    for (int t = 0; t < VW; ++t) { R0[t] = 0.0; R1[t] = 0.0; }

    if (v.geo) {
        // rows in passes of kVPass, each pass two loops over the lags (upper
        // visits, then lower visits): each hot loop holds kVPass unrolled rows
        // with the inlined weight emulation, small enough for the
        // instruction cache
        vjp_geo_rows<K, 0>(v, I, r_begin, r_end, tmax, lamlast, R0, R1, lane, T);
        if constexpr (kVPass < VW) vjp_geo_rows<K, kVPass>(v, I, r_begin, r_end, tmax, lamlast, R0, R1, lane, T);
        if constexpr (2 * kVPass < VW)
            vjp_geo_rows<K, 2 * kVPass>(v, I, r_begin, r_end, tmax, lamlast, R0, R1, lane, T);
    } else {
        // generic grid: thread `lane` owns the partner chunk [k0, k1) and walks
        // the bracket of x_m + x_k upward along it for every row of the tile
        const int span = r_end - r_begin;
        const int chunk = (span + T - 1) / T;
        const int k0 = min(r_end, r_begin + lane * chunk), k1 = min(r_end, k0 + chunk);
        const long long blast = dbits(x[n - 1]);
#pragma unroll 1
        for (int t = 0; t < tmax; ++t) {
            const int m = I + t;
            const double xm = x[m], am = v.a[m], iam = v.ia[m];
            int lo = -1;
            double r0 = 0.0, r1 = 0.0;
            for (int k = k0; k < k1; ++k) {
                const double xk = x[k];
                const double vs = xm + xk;
                double P;
                if (dbits(vs) >= blast) {
                    P = lamlast;
                } else {
                    if (lo < 0) lo = bracket_lo(x, n, vs);
                    while (dbits(x[lo + 1]) <= dbits(vs)) ++lo;
                    P = fma(vs - x[lo], D[lo], lam[lo]);
                }
                const double PN = P * N[k];
                if constexpr (K == 0) r0 += PN;
                if constexpr (K == 1) r0 = fma(PN, xm + xk, r0);
                if constexpr (K == 2) r0 = fma(PN, xm * xk, r0);
                if constexpr (K == 3 || K == 5) r0 = fma(PN, fma(am, v.ia[k], v.a[k] * iam) + 2.0, r0);
                if constexpr (K == 4 || K == 5) { const double s = am + v.a[k]; r1 = fma(PN, (s * s) * s, r1); }
            }
#pragma unroll
            for (int u = 0; u < VW; ++u)
                if (u == t) { R0[u] = r0; R1[u] = r1; }
        }
    }
#pragma unroll
    for (int t = 0; t < VW; ++t) {
        red[t * RS + lane] = R0[t];
        red[(VW + t) * RS + lane] = R1[t];
    }
    G.sync();
    // fixed-order reduction: 32-column chunks (bank-rotated), then the chunks
    const int nch = T >> 5;
    for (int w = lane; w < kVRows * nch; w += T) {
        const int r = w / nch, c = w - r * nch;
        const double* p = red + r * RS + c * 32;
        const int rot = w & 31;
        double s = 0.0;
#pragma unroll 8
        for (int q = 0; q < 32; ++q) s += p[(q + rot) & 31];
        sm.part[G.g * nch + c][r] = s;
    }
    G.sync();
    for (int r = lane; r < kVRows; r += T) {
        double s = 0.0;
        for (int c = 0; c < nch; ++c) s += sm.part[G.g * nch + c][r];
        sm.fin[G.g][r] = s;
    }
    G.sync();
}

// Row m = I + t of the task (t < tmax): its dL/dN_m contribution g and the
// parameter partials gB (beta0 or Brownian) and gS (shear); M / Lm are the
// moments of N and of lambda N.
template <int K>
__device__ __forceinline__ void vjp_tile_row(const VjpCellView& v, int m, int t, const double* fin,
                                             const double* M, const double* Lm, double b0,
                                             double bbr, double bsh, double& g, double& gB,
                                             double& gS)
{
    constexpr int VW = kVW;
    const double xm = v.x[m], am = v.a[m], iam = v.ia[m], lm = v.lam[m], Nm = v.N[m];
    double AX0 = 0.0, AX1 = 0.0;     // A for beta0 / Brownian, and for shear
    if constexpr (K <= 2) {
        double Tv = fin[t];
        if (v.geo) {
            if constexpr (K == 1) Tv = fma(xm, fin[t], fin[VW + t]);
            if constexpr (K == 2) Tv = xm * fin[t];
        }
        AX0 = Tv - fma(lm, moment_factor<K, 0>(xm, am, iam, M), moment_factor<K, 0>(xm, am, iam, Lm));
    }
    if constexpr (K == 3 || K == 5)
        AX0 = fin[t] - fma(lm, moment_factor<K, 0>(xm, am, iam, M), moment_factor<K, 0>(xm, am, iam, Lm));
    if constexpr (K == 4 || K == 5) {
        const double Tv = v.geo ? xm * fin[VW + t] : fin[VW + t];
        AX1 = Tv - fma(lm, moment_factor<K, 1>(xm, am, iam, M), moment_factor<K, 1>(xm, am, iam, Lm));
    }
    if constexpr (K <= 2) g = b0 * AX0;
    else if constexpr (K == 3) g = bbr * AX0;
    else if constexpr (K == 4) g = bsh * AX1;
    else g = fma(bbr, AX0, bsh * AX1);
    gB = 0.5 * Nm * AX0;
    gS = 0.5 * Nm * AX1;
}

} // namespace pbe_gb300
