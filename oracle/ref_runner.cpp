// =============================================================================
// oracle/ref_runner.cpp -- TEST / BASELINE INFRASTRUCTURE ONLY.
//
// Runs the reference's own CUDA kernels (built unmodified from its sources by
// oracle/build_ref.sh into oracle/_ref/*.cubin) through the CUDA driver API.
// The host side restates the reference launchers:
//   src/aggregation.cu:16-61 : n <= 0 -> InvalidValue, null -> InvalidDevicePointer,
//       M = n(n+1)/2 threads, block = block_size > 0 ? block_size : 256,
//       grid = ceil(M / block), dynamic smem = 512 doubles, kernel<F> with
//       (N, x, rhs, beta0, beta_br, beta_sh, n, log_x0, inv_log_r).
//   src/breakage.cu:14-79 : death kernel<F> (N, x, rhs, S0, v_ref, alpha, v_min, n)
//       on ceil(n / block) blocks, then birth kernel<F> (N, x, t_q, bw_q, rhs,
//       S0, v_ref, alpha, v_min, n, n_quad) on ceil(n n_quad / block) blocks
//       with 512 doubles of dynamic smem, same stream.
// Used by tests/golden/make_golden.py (golden vectors) and by
// `bench.py --impl reference` (the reference arm). Never by the library.
// =============================================================================
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>

namespace {

struct RefAggParams { int n; double log_x0; double inv_log_r; int kernel_type;
                      double beta0, beta_br, beta_sh; int block_size; };
struct RefBrkParams { int n; int n_quad; int selection; double S0, v_ref, alpha, v_min;
                      int block_size; };

CUmodule g_agg = nullptr, g_brk = nullptr;
CUfunction g_agg_k[6], g_death_k[4], g_birth_k[4];

const char* kAggNames[6] = {
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi0EEEvPKdS3_Pddddidd",
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi1EEEvPKdS3_Pddddidd",
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi2EEEvPKdS3_Pddddidd",
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi3EEEvPKdS3_Pddddidd",
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi4EEEvPKdS3_Pddddidd",
    "_ZN8pbe_cuda6detail22aggregation_rhs_kernelILi5EEEvPKdS3_Pddddidd"};
const char* kDeathNames[4] = {
    "_ZN8pbe_cuda6detail21breakage_death_kernelILi0EEEvPKdS3_Pdddddi",
    "_ZN8pbe_cuda6detail21breakage_death_kernelILi1EEEvPKdS3_Pdddddi",
    "_ZN8pbe_cuda6detail21breakage_death_kernelILi2EEEvPKdS3_Pdddddi",
    "_ZN8pbe_cuda6detail21breakage_death_kernelILi3EEEvPKdS3_Pdddddi"};
const char* kBirthNames[4] = {
    "_ZN8pbe_cuda6detail21breakage_birth_kernelILi0EEEvPKdS3_S3_S3_Pdddddii",
    "_ZN8pbe_cuda6detail21breakage_birth_kernelILi1EEEvPKdS3_S3_S3_Pdddddii",
    "_ZN8pbe_cuda6detail21breakage_birth_kernelILi2EEEvPKdS3_S3_S3_Pdddddii",
    "_ZN8pbe_cuda6detail21breakage_birth_kernelILi3EEEvPKdS3_S3_S3_Pdddddii"};

constexpr unsigned kTileBytes = 512 * sizeof(double);   // PBE_TILE * sizeof(double)

int drv(CUresult r) { return r == CUDA_SUCCESS ? 0 : 1000 + static_cast<int>(r); }

} // namespace

extern "C" {

// Loads both cubins into the current (runtime primary) context. Returns 0 on
// success, 1000 + CUresult on a driver error.
int ref_init(const char* agg_cubin, const char* brk_cubin)
{
    // Use the context the caller (the CUDA runtime, e.g. via torch) made
    // current; if none is, retain and bind the primary context of device 0.
    int rc = drv(cuInit(0));
    if (rc) return rc;
    CUcontext ctx = nullptr;
    if ((rc = drv(cuCtxGetCurrent(&ctx)))) return rc;
    if (!ctx) {
        CUdevice dev;
        if ((rc = drv(cuDeviceGet(&dev, 0)))) return rc;
        if ((rc = drv(cuDevicePrimaryCtxRetain(&ctx, dev)))) return rc;
        if ((rc = drv(cuCtxSetCurrent(ctx)))) return rc;
    }
    rc = drv(cuModuleLoad(&g_agg, agg_cubin));
    if (rc) return rc;
    rc = drv(cuModuleLoad(&g_brk, brk_cubin));
    if (rc) return rc;
    for (int f = 0; f < 6; ++f) if ((rc = drv(cuModuleGetFunction(&g_agg_k[f], g_agg, kAggNames[f])))) return rc;
    for (int f = 0; f < 4; ++f) if ((rc = drv(cuModuleGetFunction(&g_death_k[f], g_brk, kDeathNames[f])))) return rc;
    for (int f = 0; f < 4; ++f) if ((rc = drv(cuModuleGetFunction(&g_birth_k[f], g_brk, kBirthNames[f])))) return rc;
    return 0;
}

int ref_aggregation_rhs(const double* N, const double* x, double* rhs, const RefAggParams* p,
                        void* stream)
{
    if (!g_agg) return 3;   // cudaErrorInitializationError
    if (p->n <= 0) return cudaErrorInvalidValue;
    if (!N || !x || !rhs) return cudaErrorInvalidDevicePointer;
    if (p->kernel_type < 0 || p->kernel_type > 5) return cudaErrorInvalidValue;
    const long long M = static_cast<long long>(p->n) * (p->n + 1) / 2;
    const int block = (p->block_size > 0) ? p->block_size : 256;
    const long long grid = (M + block - 1) / block;
    double b0 = p->beta0, bbr = p->beta_br, bsh = p->beta_sh, lx0 = p->log_x0, ilr = p->inv_log_r;
    int n = p->n;
    void* args[] = {&N, &x, &rhs, &b0, &bbr, &bsh, &n, &lx0, &ilr};
    return drv(cuLaunchKernel(g_agg_k[p->kernel_type], static_cast<unsigned>(grid), 1, 1, block, 1, 1,
                              kTileBytes, static_cast<CUstream>(stream), args, nullptr));
}

int ref_breakage_rhs(const double* N, const double* x, const double* t_q, const double* bw_q,
                     double* rhs, const RefBrkParams* p, void* stream)
{
    if (!g_brk) return 3;
    if (p->n <= 0 || p->n_quad <= 0) return cudaErrorInvalidValue;
    if (!N || !x || !t_q || !bw_q || !rhs) return cudaErrorInvalidDevicePointer;
    if (p->selection < 0 || p->selection > 3) return cudaErrorInvalidValue;
    if (p->block_size <= 0) return cudaErrorInvalidValue;   // the reference would divide by zero
    double S0 = p->S0, vr = p->v_ref, al = p->alpha, vm = p->v_min;
    int n = p->n, nq = p->n_quad;
    const int block = p->block_size;
    const unsigned gd = static_cast<unsigned>((n + block - 1) / block);
    void* dargs[] = {&N, &x, &rhs, &S0, &vr, &al, &vm, &n};
    int rc = drv(cuLaunchKernel(g_death_k[p->selection], gd, 1, 1, block, 1, 1, 0,
                                static_cast<CUstream>(stream), dargs, nullptr));
    if (rc) return rc;
    const long long M = static_cast<long long>(n) * nq;
    const unsigned gb = static_cast<unsigned>((M + block - 1) / block);
    void* bargs[] = {&N, &x, &t_q, &bw_q, &rhs, &S0, &vr, &al, &vm, &n, &nq};
    return drv(cuLaunchKernel(g_birth_k[p->selection], gb, 1, 1, block, 1, 1, kTileBytes,
                              static_cast<CUstream>(stream), bargs, nullptr));
}

} // extern "C"
