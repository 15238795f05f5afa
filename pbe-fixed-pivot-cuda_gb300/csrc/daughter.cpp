// =============================================================================
// daughter.cpp -- host builder of the breakage daughter tables (t_q, bw_q)
// for C / Fortran / Go hosts (pbe_daughter_table in include/pbe_gb300.h).
//
// The reference documents the daughter distributions and the table
// convention -- fragment volume t_q x_j, bw_q fragments per event
// (include/pbe_cuda/breakage.cuh:43-50, docs/api.md:185-192,
// docs/theory.md:122-148) -- and builds symmetric / erosion / uniform tables
// by hand in its examples; it has no builder and no power-law table. Here:
//   symmetric binary   t = {1/2},            bw = {2}
//   erosion (eps)      t = {1 - eps, eps},   bw = {1, 1}
//   uniform            Gauss-Legendre on (0, 1), bw = 2 w
//   power law (p)      b(v|v') = (p+2) v^p / v'^(p+1) (volume constraint,
//                      docs/theory.md:34-38): Gauss-Legendre on (0, s) and
//                      (s, 1), bw = (p+2) t^p w; s = param2 (0.5 if 0).
// Gauss-Legendre nodes: Newton iteration on the three-term Legendre
// recurrence from Tricomi's initial guesses; weights 2 / ((1 - z^2) P'(z)^2).
// =============================================================================
#include <algorithm>
#include <cmath>
#include <vector>

#include "pbe_gb300.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// Gauss-Legendre rule on (a, b), nodes ascending.
void gauss_legendre(int n, double a, double b, double* t, double* w)
{
    std::vector<double> z(n), wz(n);
    for (int i = 0; i < n; ++i) {
        double x = std::cos(kPi * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = x;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = (n > 1) ? n * (x * p1 - p0) / (x * x - 1.0) : 1.0;
            const double dx = p1 / dp;
            x -= dx;
            if (std::fabs(dx) < 1e-16) break;
        }
        double p0 = 1.0, p1 = x;
        for (int k = 2; k <= n; ++k) {
            const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = (n > 1) ? n * (x * p1 - p0) / (x * x - 1.0) : 1.0;
        z[i] = x;
        wz[i] = 2.0 / ((1.0 - x * x) * dp * dp);
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int p, int q) { return z[p] < z[q]; });
    const double h = 0.5 * (b - a);
    for (int i = 0; i < n; ++i) {
        t[i] = a + h * (z[idx[i]] + 1.0);
        w[i] = h * wz[idx[i]];
    }
}

} // namespace

extern "C" int pbe_daughter_table(int kind, int order, double param, double param2, double* t_q,
                                  double* bw_q, int capacity, int* n_quad)
{
    int n = 0;
    switch (kind) {
    case PBE_DAUGHTER_SYMMETRIC: n = 1; break;
    case PBE_DAUGHTER_EROSION: n = 2; break;
    case PBE_DAUGHTER_UNIFORM: n = order; break;
    case PBE_DAUGHTER_POWERLAW: n = 2 * order; break;
    default: return 1;   // cudaErrorInvalidValue
    }
    if ((kind == PBE_DAUGHTER_UNIFORM || kind == PBE_DAUGHTER_POWERLAW) && (order < 1 || order > 512))
        return 1;
    if (kind == PBE_DAUGHTER_EROSION && !(param > 0.0 && param < 1.0)) return 1;
    const double split = (param2 == 0.0) ? 0.5 : param2;
    if (kind == PBE_DAUGHTER_POWERLAW && (!(param > -1.0) || !(split > 0.0 && split < 1.0))) return 1;
    if (n_quad) *n_quad = n;
    if (!t_q || !bw_q) return capacity == 0 ? 0 : 1;   // size query
    if (capacity < n) return 1;
    if (kind == PBE_DAUGHTER_SYMMETRIC) {
        t_q[0] = 0.5;
        bw_q[0] = 2.0;
    } else if (kind == PBE_DAUGHTER_EROSION) {
        t_q[0] = 1.0 - param; bw_q[0] = 1.0;
        t_q[1] = param;       bw_q[1] = 1.0;
    } else if (kind == PBE_DAUGHTER_UNIFORM) {
        gauss_legendre(order, 0.0, 1.0, t_q, bw_q);
        for (int i = 0; i < n; ++i) bw_q[i] *= 2.0;
    } else {
        gauss_legendre(order, 0.0, split, t_q, bw_q);
        gauss_legendre(order, split, 1.0, t_q + order, bw_q + order);
        for (int i = 0; i < n; ++i) bw_q[i] = (param + 2.0) * std::pow(t_q[i], param) * bw_q[i];
    }
    return 0;
}
