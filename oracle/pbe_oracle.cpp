// =============================================================================
// oracle/pbe_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Serial FP64 CPU restatement of the fixed-pivot population-balance RHS of
// acuoci/pbe-fixed-pivot-cuda. It is the checker for the CUDA library in this
// repository: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load it. The product never links, calls or falls back to it.
//
// Every function states the reference lines it follows (paths relative to the
// reference project). The algorithm is restated pair by pair / fragment by
// fragment in plain loops, in the reference's arithmetic order, so that the
// result differs from the reference only by summation order and by libm
// versus CUDA ulp differences in cbrt/log/pow.
//
// Besides rhs the functions can accumulate scale[i] = sum of |contribution|
// deposited into bin i (death and birth terms alike). Parity tests use it to
// define the per-bin tolerance |gpu_i - ref_i| <= tol * scale_i, which stays
// meaningful in bins where birth and death nearly cancel.
//
// Pinning: tests/test_oracle_golden.py checks these functions against rhs
// vectors produced by the reference's own CUDA kernels (built unmodified from
// its sources by oracle/build_ref.sh) and against the known-answer tests of
// tests/unit/test_aggregation.cpp and tests/unit/test_breakage.cpp.
// =============================================================================

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Aggregation frequency beta(xj, xk):
// src/aggregation_kernels.cuh:56-89 (eval_kernel_t<0..5>).
inline double beta_ref(int kernel, double xj, double xk,
                       double b0, double b_br, double b_sh)
{
    switch (kernel) {
    case 0: return b0;
    case 1: return b0 * (xj + xk);
    case 2: return b0 * xj * xk;
    case 3: {
        double xj3 = std::cbrt(xj), xk3 = std::cbrt(xk);
        return b_br * (xj3 / xk3 + xk3 / xj3 + 2.0);
    }
    case 4: {
        double s = std::cbrt(xj) + std::cbrt(xk);
        return b_sh * s * s * s;
    }
    case 5: {
        double xj3 = std::cbrt(xj), xk3 = std::cbrt(xk);
        double br = b_br * (xj3 / xk3 + xk3 / xj3 + 2.0);
        double sh = b_sh * (xj3 + xk3) * (xj3 + xk3) * (xj3 + xk3);
        return br + sh;
    }
    default: return 0.0;
    }
}

// Right bracket of v: src/aggregation_kernels.cuh:118-134 (bin_index).
// Geometric grids (inv_log_r != 0) use the logarithm formula with a clamp
// and no verification; generic grids use binary search (x[lo] <= v < x[hi]).
inline int bin_index_ref(const double* x, int n, double v,
                         double log_x0, double inv_log_r)
{
    if (inv_log_r != 0.0) {
        double pos = (std::log(v) - log_x0) * inv_log_r;
        int hi = static_cast<int>(std::floor(pos)) + 1;
        return std::min(n - 1, std::max(1, hi));
    }
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (x[mid] <= v) lo = mid; else hi = mid;
    }
    return hi;
}

// Left bracket: src/breakage_kernels.cuh:95-105 (bin_search).
inline int bin_search_ref(const double* x, int n, double v)
{
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (x[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

// Selection function: src/breakage_kernels.cuh:51-65 (eval_selection_t<0..3>).
inline double selection_ref(int sel, double v, double S0, double v_ref,
                            double alpha, double v_min)
{
    switch (sel) {
    case 0: return S0;
    case 1: return S0 * v / v_ref;
    case 2: return S0 * std::pow(v / v_ref, alpha);
    case 3: return (v > v_min) ? S0 : 0.0;
    default: return 0.0;
    }
}

inline void dep(double* rhs, double* scale, int i, double val)
{
    rhs[i] += val;
    if (scale) scale[i] += std::fabs(val);
}

// One upper-triangle row j of the aggregation sum (pairs j <= k < n):
// src/aggregation_kernels.cuh:176-231 for every k of the row.
//
// exact_bracket = 0 follows the reference literally: on a geometric grid
// (inv_log_r != 0) the bracket comes from the floating-point logarithm, which
// near a tie (v within a few ulps of a pivot) can select the neighbouring
// bracket and extrapolate (w slightly outside [0, 1]). exact_bracket = 1 uses
// the exact bracket x[lo] <= v < x[lo+1] (the reference's own generic-grid
// search, :125-132) on every grid. When `misplaced` is non-null it receives,
// per bin, |deposit(log bracket) - deposit(exact bracket)| summed over the
// pairs where the two brackets differ: the reference's own rounding noise.
void aggregation_row(const double* N, const double* x, double* rhs,
                     double* scale, double* misplaced, int n, int j,
                     double log_x0, double inv_log_r, int kernel, double b0,
                     double b_br, double b_sh, int exact_bracket)
{
    const double xj = x[j], Nj = N[j];
    for (int k = j; k < n; ++k) {
        const double xk = x[k], Nk = N[k];
        double rate = beta_ref(kernel, xj, xk, b0, b_br, b_sh) * Nj * Nk;
        const bool diagonal = (j == k);
        if (diagonal) rate *= 0.5;
        // death (:213-221)
        if (diagonal) {
            dep(rhs, scale, j, -2.0 * rate);
        } else {
            dep(rhs, scale, j, -rate);
            dep(rhs, scale, k, -rate);
        }
        // birth (:190-200, :223-231)
        const double v = xj + xk;
        if (v >= x[n - 1]) {
            dep(rhs, scale, n - 1, rate);
        } else if (v <= x[0]) {
            dep(rhs, scale, 0, rate);
        } else {
            const int hi_log = bin_index_ref(x, n, v, log_x0, inv_log_r);
            const int hi_ex = bin_index_ref(x, n, v, log_x0, 0.0);
            const int hi = exact_bracket ? hi_ex : hi_log;
            const int lo = hi - 1;
            double w = (v - x[lo]) / (x[hi] - x[lo]);
            dep(rhs, scale, lo, (1.0 - w) * rate);
            dep(rhs, scale, hi, w * rate);
            if (misplaced && hi_log != hi_ex) {
                const int h2 = exact_bracket ? hi_log : hi_ex;
                const double w2 = (v - x[h2 - 1]) / (x[h2] - x[h2 - 1]);
                // the two deposit vectors over bins {lo, hi} and {h2-1, h2}
                double d[4] = {(1.0 - w) * rate, w * rate, -(1.0 - w2) * rate, -w2 * rate};
                int b[4] = {lo, hi, h2 - 1, h2};
                for (int a = 0; a < 4; ++a) {
                    double s = 0.0;
                    bool first = true;
                    for (int c = 0; c < 4; ++c) if (b[c] == b[a]) { if (c < a) first = false; s += d[c]; }
                    if (first) misplaced[b[a]] += std::fabs(s);
                }
            }
        }
    }
}

// Row j of J(N) v for the aggregation RHS: the pairs of aggregation_row with
// the rate's derivative along v, beta (N_j v_k + v_j N_k) (times 1/2 on the
// diagonal), deposited like the rate (exact bracket).
void aggregation_row_jvp(const double* N, const double* v, const double* x, double* out,
                         double* scale, int n, int j, int kernel, double b0, double b_br,
                         double b_sh)
{
    const double xj = x[j];
    for (int k = j; k < n; ++k) {
        const double xk = x[k];
        double rate = beta_ref(kernel, xj, xk, b0, b_br, b_sh) * (N[j] * v[k] + v[j] * N[k]);
        const bool diagonal = (j == k);
        if (diagonal) rate *= 0.5;
        if (diagonal) {
            dep(out, scale, j, -2.0 * rate);
        } else {
            dep(out, scale, j, -rate);
            dep(out, scale, k, -rate);
        }
        const double vs = xj + xk;
        if (vs >= x[n - 1]) {
            dep(out, scale, n - 1, rate);
        } else if (vs <= x[0]) {
            dep(out, scale, 0, rate);
        } else {
            const int hi = bin_index_ref(x, n, vs, 0.0, 0.0);
            const int lo = hi - 1;
            const double w = (vs - x[lo]) / (x[hi] - x[lo]);
            dep(out, scale, lo, (1.0 - w) * rate);
            dep(out, scale, hi, w * rate);
        }
    }
}

// Breakage RHS (src/breakage_kernels.cuh:115-133, :160-251) of the values V
// with the guard S != 0 && G > 2.2e-308 taken on G: V = G = N is the RHS;
// G = N, V = v its Jacobian-vector product (the RHS is linear in N wherever
// the guard passes, and the guard is a property of the state).
void breakage_core(const double* G, const double* V, const double* x, const double* t_q,
                   const double* bw_q, double* rhs, double* scale, int n, int n_quad,
                   int selection, double S0, double v_ref, double alpha, double v_min)
{
    // death kernel runs first on the stream (src/breakage.cu:30-50)
    for (int j = 0; j < n; ++j) {
        double Sj = selection_ref(selection, x[j], S0, v_ref, alpha, v_min);
        if (Sj != 0.0 && G[j] > 2.2e-308) dep(rhs, scale, j, -(Sj * V[j]));
    }
    for (int j = 0; j < n; ++j) {
        const double xj = x[j], Vj = V[j];
        const double Sj = selection_ref(selection, xj, S0, v_ref, alpha, v_min);
        if (!(Sj != 0.0 && G[j] > 2.2e-308)) continue;
        for (int q = 0; q < n_quad; ++q) {
            const double contrib = Sj * Vj * bw_q[q];
            const double vf = xj * t_q[q];
            if (vf <= x[0]) {
                dep(rhs, scale, 0, contrib);
            } else if (vf >= x[n - 1]) {
                dep(rhs, scale, n - 1, contrib);
            } else {
                int lo = bin_search_ref(x, n, vf);
                int hi = lo + 1;
                double eta = (vf - x[lo]) / (x[hi] - x[lo]);
                dep(rhs, scale, lo, (1.0 - eta) * contrib);
                dep(rhs, scale, hi, eta * contrib);
            }
        }
    }
}

} // namespace

extern "C" {

// Aggregation RHS, accumulated into rhs (+=) like launch_aggregation_rhs
// (include/pbe_cuda/aggregation.cuh:115-120; kernel src/aggregation_kernels.cuh:145-239).
// scale / misplaced may be null (see aggregation_row). Returns 0, or 1 for
// n <= 0 / null pointers / bad kernel (src/aggregation.cu:23-24, :54).
int oracle_aggregation_rhs(const double* N, const double* x, double* rhs,
                           double* scale, double* misplaced, int n,
                           double log_x0, double inv_log_r, int kernel,
                           double beta0, double beta_br, double beta_sh,
                           int exact_bracket)
{
    if (n <= 0 || !N || !x || !rhs || kernel < 0 || kernel > 5) return 1;
    for (int j = 0; j < n; ++j)
        aggregation_row(N, x, rhs, scale, misplaced, n, j, log_x0, inv_log_r,
                        kernel, beta0, beta_br, beta_sh, exact_bracket);
    return 0;
}

// Same sum, rows j split over threads with thread-private rhs buffers that are
// summed in thread order at the end. Used only as the all-cores CPU baseline.
int oracle_aggregation_rhs_mt(const double* N, const double* x, double* rhs,
                              int n, double log_x0, double inv_log_r,
                              int kernel, double beta0, double beta_br,
                              double beta_sh, int nthreads)
{
    if (n <= 0 || !N || !x || !rhs || kernel < 0 || kernel > 5) return 1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    std::vector<double> priv(static_cast<size_t>(nthreads) * n, 0.0);
    #pragma omp parallel num_threads(nthreads)
    {
        const int t = omp_get_thread_num();
        double* r = priv.data() + static_cast<size_t>(t) * n;
        // rows are of unequal length (n - j): cyclic distribution balances them
        #pragma omp for schedule(dynamic, 16)
        for (int j = 0; j < n; ++j)
            aggregation_row(N, x, r, nullptr, nullptr, n, j, log_x0, inv_log_r,
                            kernel, beta0, beta_br, beta_sh, 0);
    }
    for (int t = 0; t < nthreads; ++t)
        for (int i = 0; i < n; ++i) rhs[i] += priv[static_cast<size_t>(t) * n + i];
    return 0;
#else
    (void)nthreads;
    for (int j = 0; j < n; ++j)
        aggregation_row(N, x, rhs, nullptr, nullptr, n, j, log_x0, inv_log_r,
                        kernel, beta0, beta_br, beta_sh, 0);
    return 0;
#endif
}

// Breakage RHS (+=) like launch_breakage_rhs (include/pbe_cuda/breakage.cuh:122-129).
// Death: src/breakage_kernels.cuh:115-133. Birth: :160-251. Guard
// S != 0 && N > 2.2e-308 on both (:131, :195). Returns 1 on the argument
// errors of src/breakage.cu:23-24, :46, :74.
int oracle_breakage_rhs(const double* N, const double* x, const double* t_q,
                        const double* bw_q, double* rhs, double* scale, int n,
                        int n_quad, int selection, double S0, double v_ref,
                        double alpha, double v_min)
{
    if (n <= 0 || n_quad <= 0) return 1;
    if (!N || !x || !t_q || !bw_q || !rhs) return 1;
    if (selection < 0 || selection > 3) return 1;
    breakage_core(N, N, x, t_q, bw_q, rhs, scale, n, n_quad, selection, S0, v_ref, alpha, v_min);
    return 0;
}

// J(N) v of the aggregation RHS (+= into out): aggregation_row_jvp over all
// rows. Returns 1 on the argument errors of oracle_aggregation_rhs.
int oracle_aggregation_rhs_jvp(const double* N, const double* v, const double* x, double* out,
                               double* scale, int n, int kernel, double beta0, double beta_br,
                               double beta_sh)
{
    if (n <= 0 || !N || !v || !x || !out || kernel < 0 || kernel > 5) return 1;
    for (int j = 0; j < n; ++j)
        aggregation_row_jvp(N, v, x, out, scale, n, j, kernel, beta0, beta_br, beta_sh);
    return 0;
}

// J(N) v of the breakage RHS (+= into out): breakage_core with the guard on N
// and the values v.
int oracle_breakage_rhs_jvp(const double* N, const double* v, const double* x, const double* t_q,
                            const double* bw_q, double* out, double* scale, int n, int n_quad,
                            int selection, double S0, double v_ref, double alpha, double v_min)
{
    if (n <= 0 || n_quad <= 0) return 1;
    if (!N || !v || !x || !t_q || !bw_q || !out) return 1;
    if (selection < 0 || selection > 3) return 1;
    breakage_core(N, v, x, t_q, bw_q, out, scale, n, n_quad, selection, S0, v_ref, alpha, v_min);
    return 0;
}

// Classical RK4 step on the host (examples/common/pbe_examples_utils.hpp:409-456):
// k1 = R(N), k2 = R(N + dt/2 k1), k3 = R(N + dt/2 k2), k4 = R(N + dt k3),
// N += dt/6 (k1 + 2k2 + 2k3 + k4), where R = aggregation + breakage into a
// zeroed rhs (examples/flocculation_two_stage/main.cpp:333-351). A negative
// agg_kernel skips aggregation; n_quad <= 0 skips breakage.
int oracle_rk4_step(double* N, const double* x, int n, double dt,
                    int agg_kernel, double log_x0, double inv_log_r,
                    double beta0, double beta_br, double beta_sh,
                    const double* t_q, const double* bw_q, int n_quad,
                    int selection, double S0, double v_ref, double alpha,
                    double v_min)
{
    if (n <= 0 || !N || !x) return 1;
    std::vector<double> k1(n), k2(n), k3(n), k4(n), stage(n);
    auto R = [&](const double* Nin, double* out) {
        std::fill(out, out + n, 0.0);
        if (agg_kernel >= 0)
            oracle_aggregation_rhs(Nin, x, out, nullptr, nullptr, n, log_x0,
                                   inv_log_r, agg_kernel, beta0, beta_br, beta_sh, 0);
        if (n_quad > 0)
            oracle_breakage_rhs(Nin, x, t_q, bw_q, out, nullptr, n, n_quad,
                                selection, S0, v_ref, alpha, v_min);
    };
    R(N, k1.data());
    for (int i = 0; i < n; ++i) stage[i] = N[i] + 0.5 * dt * k1[i];
    R(stage.data(), k2.data());
    for (int i = 0; i < n; ++i) stage[i] = N[i] + 0.5 * dt * k2[i];
    R(stage.data(), k3.data());
    for (int i = 0; i < n; ++i) stage[i] = N[i] + dt * k3[i];
    R(stage.data(), k4.data());
    for (int i = 0; i < n; ++i)
        N[i] += (dt / 6.0) * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
    return 0;
}

// ---------------------------------------------------------------------------
// Vector-Jacobian products (no counterpart in the reference): given
// lambda = dL/drhs, accumulate gN += dL/dN and gp += dL/d(parameters) for the
// aggregation RHS above, pair by pair. For pair p = (j <= k) with
// rate_p = c_p beta N_j N_k (c_p = 1/2 on the diagonal), L = sum_p rate_p G_p,
// G_p = P_p - lambda_j - lambda_k, P_p = (1-w) lambda_lo + w lambda_hi
// (lambda_{n-1} / lambda_0 for the clipped pairs), so
//   dL/dN_j += G_p c_p beta (1 + [j==k]) N_k ... (N_j for k), dL/dbeta_X += G_p c_p f_X N_j N_k.
// gp[0..2] = dL/dbeta0, dL/dbeta_br, dL/dbeta_sh.
// sN / sp (nullable) receive the same sums with |P| + |lambda_j| + |lambda_k|
// in place of G: the per-entry scale for relative tolerances.
int oracle_aggregation_rhs_vjp(const double* N, const double* x, const double* lam,
                               double* gN, double* gp, double* sN, double* sp, int n,
                               double log_x0, double inv_log_r, int kernel, double beta0,
                               double beta_br, double beta_sh, int exact_bracket)
{
    if (n <= 0 || !N || !x || !lam || !gN || !gp || kernel < 0 || kernel > 5) return 1;
    for (int j = 0; j < n; ++j) {
        for (int k = j; k < n; ++k) {
            const double xj = x[j], xk = x[k];
            double f0 = 0.0, fbr = 0.0, fsh = 0.0;
            if (kernel == 0) f0 = 1.0;
            if (kernel == 1) f0 = xj + xk;
            if (kernel == 2) f0 = xj * xk;
            if (kernel == 3 || kernel == 5) {
                const double a = std::cbrt(xj), b = std::cbrt(xk);
                fbr = a / b + b / a + 2.0;
            }
            if (kernel == 4 || kernel == 5) {
                const double s = std::cbrt(xj) + std::cbrt(xk);
                fsh = s * s * s;
            }
            const double beta = beta0 * f0 + beta_br * fbr + beta_sh * fsh;
            const double c = (j == k) ? 0.5 : 1.0;
            const double v = xj + xk;
            double P, Pa;
            if (v >= x[n - 1]) { P = lam[n - 1]; Pa = std::fabs(P); }
            else if (v <= x[0]) { P = lam[0]; Pa = std::fabs(P); }
            else {
                const int hi = bin_index_ref(x, n, v, log_x0, exact_bracket ? 0.0 : inv_log_r);
                const int lo = hi - 1;
                const double w = (v - x[lo]) / (x[hi] - x[lo]);
                P = (1.0 - w) * lam[lo] + w * lam[hi];
                Pa = std::fabs((1.0 - w) * lam[lo]) + std::fabs(w * lam[hi]);
            }
            const double G = P - lam[j] - lam[k];
            const double Ga = Pa + std::fabs(lam[j]) + std::fabs(lam[k]);
            if (j == k) {
                gN[j] += G * beta * N[j];
                if (sN) sN[j] += Ga * std::fabs(beta * N[j]);
            } else {
                gN[j] += G * beta * N[k];
                gN[k] += G * beta * N[j];
                if (sN) { sN[j] += Ga * std::fabs(beta * N[k]); sN[k] += Ga * std::fabs(beta * N[j]); }
            }
            const double GNN = G * c * N[j] * N[k];
            gp[0] += GNN * f0;
            gp[1] += GNN * fbr;
            gp[2] += GNN * fsh;
            if (sp) {
                const double GaNN = Ga * std::fabs(c * N[j] * N[k]);
                sp[0] += GaNN * std::fabs(f0);
                sp[1] += GaNN * std::fabs(fbr);
                sp[2] += GaNN * std::fabs(fsh);
            }
        }
    }
    return 0;
}

// Breakage VJP: rhs_i = -S_i N_i + sum_j S_j N_j sum_q bw_q eta_i(x_j t_q) over
// the guarded parents (S != 0, N > 2.2e-308). With Q_j = -lambda_j +
// sum_q bw_q P_jq: gN_j += S_j Q_j; gp[0] = dL/dS0, gp[1] = dL/dv_ref,
// gp[2] = dL/dalpha, gp[3] = dL/dv_min (0: the threshold is a step).
int oracle_breakage_rhs_vjp(const double* N, const double* x, const double* t_q,
                            const double* bw_q, const double* lam, double* gN,
                            double* gp, double* sN, double* sp, int n, int n_quad,
                            int selection, double S0, double v_ref, double alpha,
                            double v_min)
{
    if (n <= 0 || n_quad <= 0 || !N || !x || !t_q || !bw_q || !lam || !gN || !gp) return 1;
    if (selection < 0 || selection > 3) return 1;
    for (int j = 0; j < n; ++j) {
        const double xj = x[j], Nj = N[j];
        const double S = selection_ref(selection, xj, S0, v_ref, alpha, v_min);
        if (!(S != 0.0 && Nj > 2.2e-308)) continue;
        double Q = -lam[j], Qa = std::fabs(lam[j]);
        for (int q = 0; q < n_quad; ++q) {
            const double v = xj * t_q[q];
            double P, Pa;
            if (v <= x[0]) { P = lam[0]; Pa = std::fabs(P); }
            else if (v >= x[n - 1]) { P = lam[n - 1]; Pa = std::fabs(P); }
            else {
                const int lo = bin_search_ref(x, n, v);
                const double eta = (v - x[lo]) / (x[lo + 1] - x[lo]);
                P = (1.0 - eta) * lam[lo] + eta * lam[lo + 1];
                Pa = std::fabs((1.0 - eta) * lam[lo]) + std::fabs(eta * lam[lo + 1]);
            }
            Q += bw_q[q] * P;
            Qa += std::fabs(bw_q[q]) * Pa;
        }
        gN[j] += S * Q;
        if (sN) sN[j] += std::fabs(S) * Qa;
        const double NQ = Nj * Q, NQa = std::fabs(Nj) * Qa;
        gp[0] += (S / S0) * NQ;
        if (sp) sp[0] += std::fabs(S / S0) * NQa;
        if (selection == 1) { gp[1] += -(S / v_ref) * NQ; if (sp) sp[1] += std::fabs(S / v_ref) * NQa; }
        if (selection == 2) {
            gp[1] += -(alpha * S / v_ref) * NQ;
            gp[2] += S * std::log(xj / v_ref) * NQ;
            if (sp) {
                sp[1] += std::fabs(alpha * S / v_ref) * NQa;
                sp[2] += std::fabs(S * std::log(xj / v_ref)) * NQa;
            }
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Discrete adjoint of n_steps classical RK4 steps (no counterpart in the
// reference; its forward step is examples/common/pbe_examples_utils.hpp:416-456,
// restated by oracle_rk4_step above). Step s uses parameter set step_set[s]
// (NULL: set 0). agg_sets[m] = {kernel (< 0: none), beta0, beta_br, beta_sh},
// brk_sets[m] = {selection (< 0: none), S0, v_ref, alpha, v_min}. Every stage
// state of every step is kept (no checkpointing: this is the checker).
// Given lamT = dL/dN(T): NT = N(T), gN0 = dL/dN(0),
// g_agg[m][0..2] = dL/d(beta0, beta_br, beta_sh) of set m,
// g_brk[m][0..3] = dL/d(S0, v_ref, alpha, v_min) of set m.
// Per step, with h = dt/2, c = dt/6 and J_s the RHS Jacobian at stage s:
//   a4 = c lam', mu4 = J4^T a4, a3 = 2c lam' + dt mu4, mu3 = J3^T a3,
//   a2 = 2c lam' + h mu3, mu2 = J2^T a2, a1 = c lam' + h mu2, mu1 = J1^T a1,
//   lam = lam' + mu1 + mu2 + mu3 + mu4, dL/dtheta += sum_s (df/dtheta)^T a_s.
int oracle_rk4_adjoint(const double* N0, const double* x, int n, double dt, int n_steps,
                       const int* step_set, int n_sets, const double* agg_sets,
                       const double* brk_sets, const double* t_q, const double* bw_q,
                       int n_quad, const double* lamT, double* NT, double* gN0,
                       double* g_agg, double* g_brk)
{
    if (n <= 0 || n_steps < 0 || n_sets <= 0 || !N0 || !x || !lamT || !NT || !gN0) return 1;
    const size_t un = static_cast<size_t>(n);
    std::vector<double> Y(static_cast<size_t>(n_steps) * 4 * un);
    std::vector<double> N(N0, N0 + n), k(un), acc(un), st(un);
    auto set_of = [&](int s) { return step_set ? step_set[s] : 0; };
    auto R = [&](int m, const double* Nin, double* out) {
        std::fill(out, out + n, 0.0);
        const double* A = agg_sets ? agg_sets + 4 * m : nullptr;
        const double* B = brk_sets ? brk_sets + 5 * m : nullptr;
        if (A && A[0] >= 0)
            oracle_aggregation_rhs(Nin, x, out, nullptr, nullptr, n, 0.0, 0.0,
                                   static_cast<int>(A[0]), A[1], A[2], A[3], 1);
        if (B && B[0] >= 0 && n_quad > 0)
            oracle_breakage_rhs(Nin, x, t_q, bw_q, out, nullptr, n, n_quad,
                                static_cast<int>(B[0]), B[1], B[2], B[3], B[4]);
    };
    const double h = 0.5 * dt, c6 = dt / 6.0;
    const double cs[3] = {h, h, dt};
    for (int s = 0; s < n_steps; ++s) {
        const int m = set_of(s);
        double* Ys = Y.data() + static_cast<size_t>(s) * 4 * un;
        std::copy(N.begin(), N.end(), Ys);
        for (int q = 0; q < 4; ++q) {
            R(m, Ys + q * un, k.data());
            for (int i = 0; i < n; ++i) {
                acc[i] = (q == 0) ? k[i] : acc[i] + ((q == 3) ? k[i] : 2.0 * k[i]);
                if (q < 3) Ys[(q + 1) * un + i] = N[i] + cs[q] * k[i];
            }
        }
        for (int i = 0; i < n; ++i) N[i] += c6 * acc[i];
    }
    std::copy(N.begin(), N.end(), NT);
    std::vector<double> lam(lamT, lamT + n), lp(un), a(un), mu(un), lsum(un);
    if (g_agg) std::fill(g_agg, g_agg + 3 * n_sets, 0.0);
    if (g_brk) std::fill(g_brk, g_brk + 4 * n_sets, 0.0);
    std::vector<double> ga(3), gb(4);
    for (int s = n_steps - 1; s >= 0; --s) {
        const int m = set_of(s);
        const double* A = agg_sets ? agg_sets + 4 * m : nullptr;
        const double* B = brk_sets ? brk_sets + 5 * m : nullptr;
        const double* Ys = Y.data() + static_cast<size_t>(s) * 4 * un;
        lp = lam;
        lsum = lam;
        std::fill(mu.begin(), mu.end(), 0.0);
        for (int q = 3; q >= 0; --q) {
            // a_q = w_q c lam' + (coefficient of stage q+1 on k_q) mu_{q+1}
            const double w = (q == 0 || q == 3) ? c6 : 2.0 * c6;
            for (int i = 0; i < n; ++i) a[i] = (q == 3) ? w * lp[i] : w * lp[i] + cs[q] * mu[i];
            std::fill(mu.begin(), mu.end(), 0.0);
            const double* Yq = Ys + q * un;
            std::fill(ga.begin(), ga.end(), 0.0);
            std::fill(gb.begin(), gb.end(), 0.0);
            if (A && A[0] >= 0)
                oracle_aggregation_rhs_vjp(Yq, x, a.data(), mu.data(), ga.data(), nullptr, nullptr,
                                           n, 0.0, 0.0, static_cast<int>(A[0]), A[1], A[2], A[3], 1);
            if (B && B[0] >= 0 && n_quad > 0)
                oracle_breakage_rhs_vjp(Yq, x, t_q, bw_q, a.data(), mu.data(), gb.data(), nullptr,
                                        nullptr, n, n_quad, static_cast<int>(B[0]), B[1], B[2],
                                        B[3], B[4]);
            if (g_agg) for (int j = 0; j < 3; ++j) g_agg[3 * m + j] += ga[j];
            if (g_brk) for (int j = 0; j < 4; ++j) g_brk[4 * m + j] += gb[j];
            for (int i = 0; i < n; ++i) lsum[i] += mu[i];
        }
        lam = lsum;
    }
    std::copy(lam.begin(), lam.end(), gN0);
    return 0;
}

int oracle_version(void) { return 1; }

} // extern "C"
