// =============================================================================
// oracle/ref_dropin_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference's C++ API (pbe_cuda::launch_aggregation_rhs /
// launch_breakage_rhs, reference include/pbe_cuda/aggregation.cuh:115-120 and
// include/pbe_cuda/breakage.cuh:122-129) implemented on top of the reference's
// own CUDA kernels: the cubins built unmodified from its sources by
// oracle/build_ref.sh, launched by oracle/ref_runner.cpp with the reference's
// launch geometry. Linked into liboracle_ref_dropin.so together with
// ref_runner.cpp.
//
// A program written against the reference's API (its example programs) is
// linked once against libpbe_gb300.so and once against this library; the GPU
// tests run both and compare what they print, so the drop-in is checked
// against the reference's own kernels through the reference's own callers.
//
// The cubins are found in $PBE_REF_CUBIN_DIR, else in ../_ref next to this
// library's directory (oracle/_build -> oracle/_ref). They are loaded on the
// first call, into the context the CUDA runtime made current (the programs
// allocate their arrays before their first call).
//
// Like the reference's launchers the calls return cudaGetLastError() after a
// successful launch, so an earlier sticky runtime error surfaces here too.
// =============================================================================
#include <dlfcn.h>

#include <cstdlib>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "pbe_cuda/pbe_cuda.cuh"

struct RefAggParams { int n; double log_x0; double inv_log_r; int kernel_type;
                      double beta0, beta_br, beta_sh; int block_size; };
struct RefBrkParams { int n; int n_quad; int selection; double S0, v_ref, alpha, v_min;
                      int block_size; };

extern "C" int ref_init(const char* agg_cubin, const char* brk_cubin);
extern "C" int ref_aggregation_rhs(const double* N, const double* x, double* rhs,
                                   const RefAggParams* p, void* stream);
extern "C" int ref_breakage_rhs(const double* N, const double* x, const double* t_q,
                                const double* bw_q, double* rhs, const RefBrkParams* p,
                                void* stream);

namespace {

std::mutex g_mu;
bool g_ready = false;

std::string cubin_dir()
{
    if (const char* d = std::getenv("PBE_REF_CUBIN_DIR")) return d;
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&cubin_dir), &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const size_t slash = so.rfind('/');
        const std::string dir = slash == std::string::npos ? "." : so.substr(0, slash);
        return dir + "/../_ref";
    }
    return "oracle/_ref";
}

cudaError_t ensure_loaded()
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_ready) return cudaSuccess;
    // make sure the runtime's primary context exists and is current
    cudaError_t e = cudaFree(nullptr);
    if (e != cudaSuccess) return e;
    const std::string dir = cubin_dir();
    const std::string agg = dir + "/ref_aggregation.cubin";
    const std::string brk = dir + "/ref_breakage.cubin";
    if (ref_init(agg.c_str(), brk.c_str()) != 0) return cudaErrorInitializationError;
    g_ready = true;
    return cudaSuccess;
}

cudaError_t finish(int rc)
{
    if (rc >= 1000) return cudaErrorLaunchFailure;   // driver error from cuLaunchKernel
    if (rc != 0) return static_cast<cudaError_t>(rc);
    return cudaGetLastError();
}

} // namespace

namespace pbe_cuda {

cudaError_t launch_aggregation_rhs(const double* N, const double* x, double* rhs,
                                   const AggregationParams& p, cudaStream_t stream)
{
    cudaError_t e = ensure_loaded();
    if (e != cudaSuccess) return e;
    RefAggParams r{p.n, p.log_x0, p.inv_log_r, static_cast<int>(p.kernel_type), p.beta0,
                   p.beta_br, p.beta_sh, p.block_size};
    return finish(ref_aggregation_rhs(N, x, rhs, &r, stream));
}

cudaError_t launch_breakage_rhs(const double* N, const double* x, const double* t_q,
                                const double* bw_q, double* rhs, const BreakageParams& p,
                                cudaStream_t stream)
{
    cudaError_t e = ensure_loaded();
    if (e != cudaSuccess) return e;
    RefBrkParams r{p.n, p.n_quad, static_cast<int>(p.selection), p.S0, p.v_ref, p.alpha,
                   p.v_min, p.block_size};
    return finish(ref_breakage_rhs(N, x, t_q, bw_q, rhs, &r, stream));
}

} // namespace pbe_cuda
