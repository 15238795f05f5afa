// =============================================================================
// noalloc.cu -- aggregation RHS entry point that allocates no memory.
//
// Some host codes cannot let a library allocate device memory: a CFD or ODE
// solver that hands the whole GPU to its own allocator at start-up, a code
// that forbids any allocation once time stepping has begun (to keep a fixed
// memory footprint and no allocator latency inside the step), or a plug-in
// interface that can pass only the state arrays and has no way to thread a
// workspace buffer through. pbe_aggregation_rhs_noalloc serves them: it runs
// the same aggregation kernels as pbe_aggregation_rhs, but its scratch is the
// file-scope device array below, which the library image carries and which
// every GPU that loads the library holds until the process exits.
//
// Limit: n <= kNoAllocMaxN (32768 bins, about 8.5 MiB of scratch); larger n
// returns cudaErrorInvalidValue without launching anything.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress; in host code the
// array's name is only a host-side stand-in and must never be handed to a
// kernel. Make that first call before any stream capture begins. If the
// look-up fails, the call returns its error and the next call tries again.
//
// Sharing: every call on a device uses the same array and it keeps the last
// call's contents. Each call's own kernels rewrite everything they read
// (tables, moment partials, clip partials) and reset the task counter before
// use, so no clearing is needed between calls -- but calls whose kernels
// overlap on the GPU (different streams, no ordering between them) race on
// the array and give wrong results. Order such calls on one stream.
//
// The call makes no cudaMalloc / cudaFree / pool or other allocating call.
// =============================================================================
#include <mutex>

#include "pbe_internal.cuh"
#include "pbe_gb300.h"

namespace pbe_gb300 {
namespace {

constexpr int kNoAllocMaxN = 32768;
constexpr size_t kNoAllocBytes = agg_ws_bytes(kNoAllocMaxN);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
struct NoAllocDevice {
    std::mutex mu;
    bool ready = false;        // set only once the look-up below has succeeded
    void* scratch = nullptr;   // device address of g_noalloc_scratch on this device
    int num_sms = 0;
};
NoAllocDevice g_na[kMaxDevices];

// The argument checks of pbe_aggregation_rhs, in the same order (reference
// src/aggregation.cu:23-24, :54): n, pointers, enum, block_size.
cudaError_t check_args(const double* N, const double* x, const double* rhs,
                       const pbe_agg_params_t* p)
{
    if (!p) return cudaErrorInvalidValue;
    if (p->n <= 0) return cudaErrorInvalidValue;
    if (!N || !x || !rhs) return cudaErrorInvalidDevicePointer;
    if (p->kernel_type < 0 || p->kernel_type > 5) return cudaErrorInvalidValue;
    if (p->block_size > 1024) return cudaErrorInvalidConfiguration;
    return cudaSuccess;
}

} // namespace
} // namespace pbe_gb300

using namespace pbe_gb300;

extern "C" int pbe_aggregation_rhs_noalloc(const double* N, const double* x, double* rhs,
                                           const pbe_agg_params_t* params, int mode,
                                           void* stream)
{
    cudaError_t e = check_args(N, x, rhs, params);
    if (e != cudaSuccess) return e;
    if (params->n > kNoAllocMaxN) return cudaErrorInvalidValue;
    if (agg_ws_layout(params->n, nullptr, nullptr) > kNoAllocBytes) return cudaErrorInvalidValue;

    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    NoAllocDevice& st = g_na[dev];
    {
        // A failed look-up is not remembered: the next call retries it.
        std::lock_guard<std::mutex> lock(st.mu);
        if (!st.ready) {
            void* p = nullptr;
            int sms = 0;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            st.scratch = p;
            st.num_sms = sms;
            st.ready = true;
        }
    }

    AggArgs a{N, x, rhs, params->n, params->kernel_type, params->beta0, params->beta_br,
              params->beta_sh};
    return agg_launch(a, mode_is_scatter(mode), st.scratch, st.num_sms,
                      static_cast<cudaStream_t>(stream));
}
