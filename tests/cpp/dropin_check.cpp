// tests/cpp/dropin_check.cpp -- compiled by tests/test_gpu_cpp_dropin.py with
// the host C++ compiler against include/ and libpbe_gb300.so, the way a C++
// ODE/CFD host that used the reference's API would build.
//
// Checks, through compiled C++ callers:
//   * pbe_cuda::launch_aggregation_rhs / launch_breakage_rhs (the reference's
//     signatures, default stream argument) give bitwise the same rhs as the C
//     ABI's pbe_aggregation_rhs_ex / pbe_breakage_rhs_ex in gather mode, for
//     every aggregation kernel and selection function, accumulating into a
//     non-zero rhs as the reference's contract allows;
//   * the VJP entry points of both interfaces agree bitwise;
//   * the C++ calls return the reference's error codes (n <= 0 ->
//     cudaErrorInvalidValue, null -> cudaErrorInvalidDevicePointer, unknown
//     enum -> cudaErrorInvalidValue; reference src/aggregation.cu:23-24, :54,
//     src/breakage.cu:23-24, :46);
//   * a C++ struct passed through a pointer cast reaches the C ABI intact.
// Prints one line per check and "ALL OK" at the end; exit status 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "pbe_cuda/pbe_cuda.cuh"
#include "pbe_gb300.h"

namespace {

int g_fail = 0;

void expect(bool ok, const char* what)
{
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    if (!ok) ++g_fail;
}

#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            std::printf("FAIL %s -> %s\n", #call, cudaGetErrorString(e_));           \
            std::exit(2);                                                            \
        }                                                                            \
    } while (0)

struct Dev {
    double* p = nullptr;
    size_t n = 0;
    explicit Dev(size_t n_) : n(n_) { CK(cudaMalloc(&p, n * sizeof(double))); }
    ~Dev() { cudaFree(p); }
    void put(const std::vector<double>& h) { CK(cudaMemcpy(p, h.data(), n * sizeof(double), cudaMemcpyHostToDevice)); }
    std::vector<double> get() const
    {
        std::vector<double> h(n);
        CK(cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
        return h;
    }
};

bool same_bits(const std::vector<double>& a, const std::vector<double>& b)
{
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(double)) == 0;
}

} // namespace

int main()
{
    const int n = 1500;
    // geometric grid x_i = 1e-21 2^(i/64), lognormal N around bin 400
    std::vector<double> x(n), N(n), base(n);
    for (int i = 0; i < n; ++i) {
        x[i] = 1e-21 * std::pow(2.0, i / 64.0);
        const double z = (i - 400) / 90.0;
        N[i] = 1e12 * std::exp(-0.5 * z * z);
        base[i] = 1e3 * std::sin(0.37 * i);   // rhs holds other source terms already
    }
    const int nq = 8;
    std::vector<double> tq(nq), bw(nq);
    for (int q = 0; q < nq; ++q) { tq[q] = (q + 0.5) / nq; bw[q] = 2.0 / nq; }

    Dev dN(n), dx(n), dt(nq), db(nq), r1(n), r2(n), lam(n), g1(n), g2(n), gp1(4), gp2(4);
    dN.put(N); dx.put(x); dt.put(tq); db.put(bw);
    std::vector<double> lam_h(n);
    for (int i = 0; i < n; ++i) lam_h[i] = std::cos(0.11 * i);
    lam.put(lam_h);

    const char* agg_names[6] = {"Constant", "Sum", "Product", "Brownian", "Shear", "BrownianShear"};
    for (int k = 0; k < 6; ++k) {
        pbe_cuda::AggregationParams p;
        p.n = n;
        p.log_x0 = std::log(x[0]);
        p.inv_log_r = 1.0 / std::log(x[1] / x[0]);
        p.kernel_type = static_cast<pbe_cuda::AggregationKernel>(k);
        p.beta0 = k == 1 ? 1e3 : (k == 2 ? 1e21 : 1e-16);
        p.beta_br = 6.73e-18;
        p.beta_sh = 4.0 * 50.0 / 3.0;
        r1.put(base); r2.put(base);
        CK(pbe_cuda::launch_aggregation_rhs(dN.p, dx.p, r1.p, p));
        CK(static_cast<cudaError_t>(pbe_aggregation_rhs_ex(
            dN.p, dx.p, r2.p, reinterpret_cast<const pbe_agg_params_t*>(&p), PBE_MODE_GATHER,
            nullptr, 0, nullptr)));
        CK(cudaDeviceSynchronize());
        char what[160];
        std::snprintf(what, sizeof what, "aggregation %-13s C++ == C ABI (gather), bitwise", agg_names[k]);
        expect(same_bits(r1.get(), r2.get()), what);

        std::vector<double> zero(n, 0.0), z4(4, 0.0);
        g1.put(zero); g2.put(zero); gp1.put(z4); gp2.put(z4);
        CK(pbe_cuda::launch_aggregation_rhs_vjp(dN.p, dx.p, lam.p, g1.p, gp1.p, p));
        pbe_agg_params_t c;
        std::memcpy(&c, &p, sizeof c);
        CK(static_cast<cudaError_t>(pbe_aggregation_rhs_vjp(dN.p, dx.p, lam.p, g2.p, gp2.p, &c,
                                                             nullptr, 0, nullptr)));
        CK(cudaDeviceSynchronize());
        std::snprintf(what, sizeof what, "aggregation %-13s VJP C++ == C ABI, bitwise", agg_names[k]);
        expect(same_bits(g1.get(), g2.get()) && same_bits(gp1.get(), gp2.get()), what);
    }

    const char* sel_names[4] = {"Constant", "Linear", "PowerLaw", "Threshold"};
    for (int s = 0; s < 4; ++s) {
        pbe_cuda::BreakageParams p;
        p.n = n;
        p.n_quad = nq;
        p.selection = static_cast<pbe_cuda::BreakageSelection>(s);
        p.S0 = 1e-3;
        p.v_ref = x[n / 2];
        p.alpha = 0.8;
        p.v_min = x[700];
        r1.put(base); r2.put(base);
        CK(pbe_cuda::launch_breakage_rhs(dN.p, dx.p, dt.p, db.p, r1.p, p));
        CK(static_cast<cudaError_t>(pbe_breakage_rhs_ex(
            dN.p, dx.p, dt.p, db.p, r2.p, reinterpret_cast<const pbe_brk_params_t*>(&p),
            PBE_MODE_GATHER, nullptr, 0, nullptr)));
        CK(cudaDeviceSynchronize());
        char what[160];
        std::snprintf(what, sizeof what, "breakage %-9s C++ == C ABI (gather), bitwise", sel_names[s]);
        expect(same_bits(r1.get(), r2.get()), what);

        std::vector<double> zero(n, 0.0), z4(4, 0.0);
        g1.put(zero); g2.put(zero); gp1.put(z4); gp2.put(z4);
        CK(pbe_cuda::launch_breakage_rhs_vjp(dN.p, dx.p, dt.p, db.p, lam.p, g1.p, gp1.p, p));
        pbe_brk_params_t c;
        std::memcpy(&c, &p, sizeof c);
        CK(static_cast<cudaError_t>(pbe_breakage_rhs_vjp(dN.p, dx.p, dt.p, db.p, lam.p, g2.p,
                                                         gp2.p, &c, nullptr, 0, nullptr)));
        CK(cudaDeviceSynchronize());
        std::snprintf(what, sizeof what, "breakage %-9s VJP C++ == C ABI, bitwise", sel_names[s]);
        expect(same_bits(g1.get(), g2.get()) && same_bits(gp1.get(), gp2.get()), what);
    }

    // reference error codes through the C++ API
    {
        pbe_cuda::AggregationParams p;
        p.n = 0;
        expect(pbe_cuda::launch_aggregation_rhs(dN.p, dx.p, r1.p, p) == cudaErrorInvalidValue,
               "aggregation n = 0 -> cudaErrorInvalidValue");
        p.n = n;
        expect(pbe_cuda::launch_aggregation_rhs(nullptr, dx.p, r1.p, p) == cudaErrorInvalidDevicePointer,
               "aggregation N = null -> cudaErrorInvalidDevicePointer");
        p.kernel_type = static_cast<pbe_cuda::AggregationKernel>(9);
        expect(pbe_cuda::launch_aggregation_rhs(dN.p, dx.p, r1.p, p) == cudaErrorInvalidValue,
               "aggregation kernel_type 9 -> cudaErrorInvalidValue");
        pbe_cuda::BreakageParams b;
        b.n = n;
        b.n_quad = 0;
        expect(pbe_cuda::launch_breakage_rhs(dN.p, dx.p, dt.p, db.p, r1.p, b) == cudaErrorInvalidValue,
               "breakage n_quad = 0 -> cudaErrorInvalidValue");
        b.n_quad = nq;
        expect(pbe_cuda::launch_breakage_rhs(dN.p, dx.p, nullptr, db.p, r1.p, b) ==
                   cudaErrorInvalidDevicePointer,
               "breakage t_q = null -> cudaErrorInvalidDevicePointer");
        b.selection = static_cast<pbe_cuda::BreakageSelection>(-1);
        expect(pbe_cuda::launch_breakage_rhs(dN.p, dx.p, dt.p, db.p, r1.p, b) == cudaErrorInvalidValue,
               "breakage selection -1 -> cudaErrorInvalidValue");
    }
    // defaults of the reference's structs
    {
        pbe_cuda::AggregationParams a;
        pbe_cuda::BreakageParams b;
        expect(a.n == 0 && a.kernel_type == pbe_cuda::AggregationKernel::Constant && a.beta0 == 1.0 &&
                   a.beta_br == 0.0 && a.beta_sh == 0.0 && a.block_size == 256,
               "AggregationParams defaults");
        expect(b.n == 0 && b.n_quad == 0 && b.selection == pbe_cuda::BreakageSelection::Constant &&
                   b.S0 == 1.0 && b.v_ref == 1.0 && b.alpha == 1.0 && b.v_min == 0.0 &&
                   b.block_size == 256,
               "BreakageParams defaults");
    }
    if (g_fail) {
        std::printf("%d FAILED\n", g_fail);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
