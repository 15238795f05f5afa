// =============================================================================
// api.cu -- argument checking, scratch management and the two public faces of
// libpbe_gb300: the C ABI (include/pbe_gb300.h) and the C++ drop-in API
// (include/pbe_cuda/*.cuh, same signatures as acuoci/pbe-fixed-pivot-cuda).
//
// Error behaviour follows the reference launchers (src/aggregation.cu:23-24,
// :54, :60; src/breakage.cu:23-24, :46, :49, :74, :77): n <= 0 (n_quad <= 0)
// and unknown enums -> cudaErrorInvalidValue, null pointers ->
// cudaErrorInvalidDevicePointer, otherwise cudaGetLastError() after the
// launches. Two deliberate differences: breakage block_size <= 0 is rejected
// with cudaErrorInvalidValue (the reference divides by it on the host), and a
// block_size above 1024 is rejected up front with
// cudaErrorInvalidConfiguration (the reference gets the same code from the
// failed launch).
//
// Scratch: the drop-in calls take their scratch from a library-private CUDA
// memory pool per device with stream-ordered allocation
// (cudaMallocFromPoolAsync / cudaFreeAsync on the caller's stream), so
// concurrent calls on different streams never share scratch and the calls
// stay legal inside CUDA stream capture. The pool keeps freed memory
// (release threshold = max) so steady-state calls do not reach the driver.
// =============================================================================
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cstddef>
#include <type_traits>

#include "pbe_internal.cuh"
#include "pbe_gb300.h"
#include "pbe_cuda/pbe_cuda.cuh"

namespace pbe_gb300 {
namespace {

constexpr int kMaxDevices = 64;

struct DeviceState {
    std::mutex mu;
    bool ready = false;           // set only once the set-up below has succeeded
    cudaMemPool_t pool = nullptr;
    int num_sms = 0;
};
DeviceState g_dev[kMaxDevices];

// Per-device set-up (SM count, the scratch pool). A failed attempt is not
// remembered: it is released and the next call tries again, so one failure
// (for instance a first call made inside stream capture) does not poison the
// device for the rest of the process.
cudaError_t device_state(DeviceState** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    DeviceState& st = g_dev[dev];
    std::lock_guard<std::mutex> lock(st.mu);
    if (!st.ready) {
        int sms = 0;
        cudaMemPool_t pool = nullptr;
        cudaError_t err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (err == cudaSuccess) {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            err = cudaMemPoolCreate(&pool, &props);
        }
        if (err == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            err = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        if (err != cudaSuccess) {
            if (pool) cudaMemPoolDestroy(pool);
            return err;
        }
        st.num_sms = sms;
        st.pool = pool;
        st.ready = true;
    }
    *out = &st;
    return cudaSuccess;
}

int resolve_mode(int mode)
{
    if (mode == PBE_MODE_SCATTER || mode == PBE_MODE_GATHER) return mode;
    static int env_mode = []() {
        const char* s = std::getenv("PBE_GB300_MODE");
        return (s && std::strcmp(s, "scatter") == 0) ? PBE_MODE_SCATTER : PBE_MODE_GATHER;
    }();
    return env_mode;
}

// Runs `launch(ws)` with caller scratch (if given and large enough) or with a
// stream-ordered pool allocation released on the same stream afterwards.
template <class Fn>
cudaError_t with_scratch(size_t need, void* ws, size_t ws_bytes, cudaStream_t s, DeviceState* st,
                         Fn&& launch)
{
    if (need == 0) return launch(nullptr);
    if (ws) {
        if (ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 255u) != 0)
            return cudaErrorInvalidValue;
        return launch(ws);
    }
    void* p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, need, st->pool, s);
    if (e != cudaSuccess) return e;
    cudaError_t le = launch(p);
    cudaError_t fe = cudaFreeAsync(p, s);
    return le != cudaSuccess ? le : fe;
}

cudaError_t check_agg(const double* N, const double* x, double* rhs, const pbe_agg_params_t* p)
{
    if (!p) return cudaErrorInvalidValue;
    if (p->n <= 0) return cudaErrorInvalidValue;
    if (!N || !x || !rhs) return cudaErrorInvalidDevicePointer;
    if (p->kernel_type < 0 || p->kernel_type > 5) return cudaErrorInvalidValue;
    if (p->block_size > 1024) return cudaErrorInvalidConfiguration;
    return cudaSuccess;
}

cudaError_t check_brk(const double* N, const double* x, const double* t_q, const double* bw_q,
                      double* rhs, const pbe_brk_params_t* p)
{
    if (!p) return cudaErrorInvalidValue;
    if (p->n <= 0 || p->n_quad <= 0) return cudaErrorInvalidValue;
    if (!N || !x || !t_q || !bw_q || !rhs) return cudaErrorInvalidDevicePointer;
    if (p->selection < 0 || p->selection > 3) return cudaErrorInvalidValue;
    if (p->block_size <= 0) return cudaErrorInvalidValue;
    if (p->block_size > 1024) return cudaErrorInvalidConfiguration;
    if (static_cast<long long>(p->n) * p->n_quad > 0x7fffffffLL) return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t agg_call(const double* N, const double* x, double* rhs, const pbe_agg_params_t* p,
                     int mode, void* ws, size_t ws_bytes, cudaStream_t s)
{
    cudaError_t e = check_agg(N, x, rhs, p);
    if (e != cudaSuccess) return e;
    DeviceState* st = nullptr;
    e = device_state(&st);
    if (e != cudaSuccess) return e;
    const bool scatter = resolve_mode(mode) == PBE_MODE_SCATTER;
    AggArgs a{N, x, rhs, p->n, p->kernel_type, p->beta0, p->beta_br, p->beta_sh};
    const size_t need = agg_ws_layout(p->n, nullptr, nullptr);
    return with_scratch(need, ws, ws_bytes, s, st, [&](void* w) {
        return agg_launch(a, scatter, w, st->num_sms, s);
    });
}

cudaError_t brk_call(const double* N, const double* x, const double* t_q, const double* bw_q,
                     double* rhs, const pbe_brk_params_t* p, int mode, void* ws, size_t ws_bytes,
                     cudaStream_t s)
{
    cudaError_t e = check_brk(N, x, t_q, bw_q, rhs, p);
    if (e != cudaSuccess) return e;
    DeviceState* st = nullptr;
    e = device_state(&st);
    if (e != cudaSuccess) return e;
    const bool scatter = resolve_mode(mode) == PBE_MODE_SCATTER;
    BrkArgs a{N, x, t_q, bw_q, rhs, p->n, p->n_quad, p->selection, p->S0, p->v_ref, p->alpha, p->v_min};
    const size_t need = scatter ? 0 : brk_ws_layout(p->n, p->n_quad, nullptr, nullptr);
    return with_scratch(need, ws, ws_bytes, s, st, [&](void* w) {
        return brk_launch(a, scatter, w, s);
    });
}

cudaError_t agg_vjp_call(const double* N, const double* x, const double* lam, double* gN,
                         double* gp, const pbe_agg_params_t* p, void* ws, size_t ws_bytes,
                         cudaStream_t s)
{
    cudaError_t e = check_agg(N, x, gN, p);
    if (e != cudaSuccess) return e;
    if (!lam || !gp) return cudaErrorInvalidDevicePointer;
    DeviceState* st = nullptr;
    e = device_state(&st);
    if (e != cudaSuccess) return e;
    AggVjpArgs a{N, x, lam, gN, gp, p->n, p->kernel_type, p->beta0, p->beta_br, p->beta_sh};
    const size_t need = vjp_ws_layout(p->n, nullptr, nullptr);
    return with_scratch(need, ws, ws_bytes, s, st, [&](void* w) {
        return agg_vjp_launch(a, w, st->num_sms, s);
    });
}

cudaError_t brk_vjp_call(const double* N, const double* x, const double* t_q, const double* bw_q,
                         const double* lam, double* gN, double* gp, const pbe_brk_params_t* p,
                         void* ws, size_t ws_bytes, cudaStream_t s)
{
    cudaError_t e = check_brk(N, x, t_q, bw_q, gN, p);
    if (e != cudaSuccess) return e;
    if (!lam || !gp) return cudaErrorInvalidDevicePointer;
    DeviceState* st = nullptr;
    e = device_state(&st);
    if (e != cudaSuccess) return e;
    BrkVjpArgs a{N, x, t_q, bw_q, lam, gN, gp, p->n, p->n_quad, p->selection, p->S0, p->v_ref,
                 p->alpha, p->v_min};
    const size_t need = vjp_ws_layout(p->n, nullptr, nullptr);
    return with_scratch(need, ws, ws_bytes, s, st, [&](void* w) {
        return brk_vjp_launch(a, w, s);
    });
}

} // namespace

bool mode_is_scatter(int mode) { return resolve_mode(mode) == PBE_MODE_SCATTER; }

} // namespace pbe_gb300

using namespace pbe_gb300;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int pbe_aggregation_rhs(const double* N, const double* x, double* rhs,
                        const pbe_agg_params_t* params, void* stream)
{
    return static_cast<int>(agg_call(N, x, rhs, params, PBE_MODE_DEFAULT, nullptr, 0,
                                     static_cast<cudaStream_t>(stream)));
}

int pbe_breakage_rhs(const double* N, const double* x, const double* t_q, const double* bw_q,
                     double* rhs, const pbe_brk_params_t* params, void* stream)
{
    return static_cast<int>(brk_call(N, x, t_q, bw_q, rhs, params, PBE_MODE_DEFAULT, nullptr, 0,
                                     static_cast<cudaStream_t>(stream)));
}

size_t pbe_aggregation_workspace_bytes(int n, int mode)
{
    (void)mode;
    if (n <= 0) return 0;
    return agg_ws_layout(n, nullptr, nullptr);
}

size_t pbe_breakage_workspace_bytes(int n, int n_quad, int mode)
{
    if (n <= 0 || n_quad <= 0) return 0;
    if (resolve_mode(mode) == PBE_MODE_SCATTER) return 0;
    return brk_ws_layout(n, n_quad, nullptr, nullptr);
}

int pbe_aggregation_rhs_ex(const double* N, const double* x, double* rhs,
                           const pbe_agg_params_t* params, int mode, void* workspace,
                           size_t workspace_bytes, void* stream)
{
    return static_cast<int>(agg_call(N, x, rhs, params, mode, workspace, workspace_bytes,
                                     static_cast<cudaStream_t>(stream)));
}

int pbe_breakage_rhs_ex(const double* N, const double* x, const double* t_q, const double* bw_q,
                        double* rhs, const pbe_brk_params_t* params, int mode, void* workspace,
                        size_t workspace_bytes, void* stream)
{
    return static_cast<int>(brk_call(N, x, t_q, bw_q, rhs, params, mode, workspace,
                                     workspace_bytes, static_cast<cudaStream_t>(stream)));
}

const char* pbe_error_string(int code)
{
    return cudaGetErrorString(static_cast<cudaError_t>(code));
}

int pbe_version(void) { return 100; }

size_t pbe_vjp_workspace_bytes(int n)
{
    if (n <= 0) return 0;
    return vjp_ws_layout(n, nullptr, nullptr);
}

int pbe_aggregation_rhs_vjp(const double* N, const double* x, const double* lambda, double* gN,
                            double* gparams, const pbe_agg_params_t* params, void* workspace,
                            size_t workspace_bytes, void* stream)
{
    return static_cast<int>(agg_vjp_call(N, x, lambda, gN, gparams, params, workspace,
                                         workspace_bytes, static_cast<cudaStream_t>(stream)));
}

int pbe_breakage_rhs_vjp(const double* N, const double* x, const double* t_q, const double* bw_q,
                         const double* lambda, double* gN, double* gparams,
                         const pbe_brk_params_t* params, void* workspace, size_t workspace_bytes,
                         void* stream)
{
    return static_cast<int>(brk_vjp_call(N, x, t_q, bw_q, lambda, gN, gparams, params, workspace,
                                         workspace_bytes, static_cast<cudaStream_t>(stream)));
}

int pbe_scratch_pool_usage(unsigned long long* reserved_bytes, unsigned long long* used_high_bytes,
                           int reset_high)
{
    if (!reserved_bytes || !used_high_bytes) return cudaErrorInvalidValue;
    *reserved_bytes = 0;
    *used_high_bytes = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    DeviceState& st = g_dev[dev];
    std::lock_guard<std::mutex> lock(st.mu);
    if (!st.ready) return cudaSuccess;   // no pool yet: nothing was ever allocated from it
    unsigned long long v = 0;
    e = cudaMemPoolGetAttribute(st.pool, cudaMemPoolAttrReservedMemCurrent, &v);
    if (e != cudaSuccess) return e;
    *reserved_bytes = v;
    e = cudaMemPoolGetAttribute(st.pool, cudaMemPoolAttrUsedMemHigh, &v);
    if (e != cudaSuccess) return e;
    *used_high_bytes = v;
    if (reset_high) {
        unsigned long long zero = 0;
        e = cudaMemPoolSetAttribute(st.pool, cudaMemPoolAttrUsedMemHigh, &zero);
    }
    return e;
}

int pbe_set_profile_events(void* start, void* stop)
{
    g_prof_start = static_cast<cudaEvent_t>(start);
    g_prof_stop = static_cast<cudaEvent_t>(stop);
    return 0;
}

} // extern "C"

// ---------------------------------------------------------------------------
// C++ drop-in API (pbe_cuda namespace, reference signatures)
// ---------------------------------------------------------------------------
// The C structs and the C++ structs must share their layout member by member,
// so a caller may pass either through the other interface.
#define PBE_SAME_MEMBER(CPP, C, m)                                                     \
    static_assert(offsetof(pbe_cuda::CPP, m) == offsetof(C, m) &&                      \
                      sizeof(pbe_cuda::CPP::m) == sizeof(((C*)nullptr)->m),            \
                  #CPP "::" #m " and " #C "." #m " differ in offset or size")
static_assert(sizeof(pbe_cuda::AggregationParams) == sizeof(pbe_agg_params_t),
              "AggregationParams and pbe_agg_params_t must share their layout");
static_assert(sizeof(pbe_cuda::BreakageParams) == sizeof(pbe_brk_params_t),
              "BreakageParams and pbe_brk_params_t must share their layout");
static_assert(std::is_standard_layout<pbe_cuda::AggregationParams>::value &&
                  std::is_standard_layout<pbe_cuda::BreakageParams>::value,
              "the C++ parameter structs must be standard-layout");
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, n);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, log_x0);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, inv_log_r);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, kernel_type);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, beta0);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, beta_br);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, beta_sh);
PBE_SAME_MEMBER(AggregationParams, pbe_agg_params_t, block_size);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, n);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, n_quad);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, selection);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, S0);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, v_ref);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, alpha);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, v_min);
PBE_SAME_MEMBER(BreakageParams, pbe_brk_params_t, block_size);
#undef PBE_SAME_MEMBER

namespace pbe_cuda {

cudaError_t launch_aggregation_rhs(const double* N, const double* x, double* rhs,
                                   const AggregationParams& p, cudaStream_t stream)
{
    pbe_agg_params_t c;
    c.n = p.n; c.log_x0 = p.log_x0; c.inv_log_r = p.inv_log_r;
    c.kernel_type = static_cast<int>(p.kernel_type);
    c.beta0 = p.beta0; c.beta_br = p.beta_br; c.beta_sh = p.beta_sh;
    c.block_size = p.block_size;
    return agg_call(N, x, rhs, &c, PBE_MODE_DEFAULT, nullptr, 0, stream);
}

cudaError_t launch_breakage_rhs(const double* N, const double* x, const double* t_q,
                                const double* bw_q, double* rhs, const BreakageParams& p,
                                cudaStream_t stream)
{
    pbe_brk_params_t c;
    c.n = p.n; c.n_quad = p.n_quad; c.selection = static_cast<int>(p.selection);
    c.S0 = p.S0; c.v_ref = p.v_ref; c.alpha = p.alpha; c.v_min = p.v_min;
    c.block_size = p.block_size;
    return brk_call(N, x, t_q, bw_q, rhs, &c, PBE_MODE_DEFAULT, nullptr, 0, stream);
}

cudaError_t launch_aggregation_rhs_vjp(const double* N, const double* x, const double* lambda,
                                       double* gN, double* gparams, const AggregationParams& p,
                                       cudaStream_t stream)
{
    pbe_agg_params_t c;
    c.n = p.n; c.log_x0 = p.log_x0; c.inv_log_r = p.inv_log_r;
    c.kernel_type = static_cast<int>(p.kernel_type);
    c.beta0 = p.beta0; c.beta_br = p.beta_br; c.beta_sh = p.beta_sh;
    c.block_size = p.block_size;
    return agg_vjp_call(N, x, lambda, gN, gparams, &c, nullptr, 0, stream);
}

cudaError_t launch_breakage_rhs_vjp(const double* N, const double* x, const double* t_q,
                                    const double* bw_q, const double* lambda, double* gN,
                                    double* gparams, const BreakageParams& p, cudaStream_t stream)
{
    pbe_brk_params_t c;
    c.n = p.n; c.n_quad = p.n_quad; c.selection = static_cast<int>(p.selection);
    c.S0 = p.S0; c.v_ref = p.v_ref; c.alpha = p.alpha; c.v_min = p.v_min;
    c.block_size = p.block_size;
    return brk_vjp_call(N, x, t_q, bw_q, lambda, gN, gparams, &c, nullptr, 0, stream);
}

} // namespace pbe_cuda
