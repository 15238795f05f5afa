// =============================================================================
// batch_vjp.cu -- vector-Jacobian products of the batched RHS and the
// elementwise steps of the batched RK4 adjoint (sm_103a, FP64).
//
// Given lambda = dL/drhs for every cell (packed like N), one VJP is three
// launches:
//  * batch_vjp_prep_kernel, one CTA per cell: x N and the lambda slopes
//    D_i = (lambda_{i+1} - lambda_i) / (x_{i+1} - x_i), the moments of N and of
//    lambda N (the -lambda_j - lambda_k part of the aggregation adjoint), and
//    the whole breakage VJP of the cell (per parent: Q_j = -lambda_j +
//    sum_q bw_q P_jq from the grid's fragment tables, gN_j += S_j Q_j, and the
//    cell's dL/dS0, dL/dv_ref, dL/dalpha);
//  * batch_vjp_main_kernel, persistent over bundles of row-tile tasks (cell,
//    first row), running the shared row-tile body (vjp_tile.cuh) on groups of
//    T threads; each task adds its rows' dL/dN and stores its parameter
//    partials at a fixed slot of its cell;
//  * batch_vjp_gfin_kernel, one thread per cell: the cell's partials in tile
//    order -> dL/dbeta. Every sum has a fixed order: deterministic.
// The per-lag tables are the forward's (beta-free, 1/2 on lag 0, so the VJP
// scales lag 0 by 2).
// =============================================================================
#include "batch_internal.cuh"
#include "vjp_tile.cuh"

namespace pbe_gb300 {
namespace {

constexpr int VW = kVW;

__device__ __forceinline__ double sel_value_v(int F, double v, double S0, double v_ref,
                                              double alpha, double v_min)
{
    switch (F) {
    case 0: return selection<0>(v, S0, v_ref, alpha, v_min);
    case 1: return selection<1>(v, S0, v_ref, alpha, v_min);
    case 2: return selection<2>(v, S0, v_ref, alpha, v_min);
    default: return selection<3>(v, S0, v_ref, alpha, v_min);
    }
}

__global__ void __launch_bounds__(256)
batch_vjp_prep_kernel(BatchDev d, BatchVjpDev vd, const double* __restrict__ N,
                      const double* __restrict__ lam, double* __restrict__ gN,
                      double* __restrict__ gparams, const pbe_batch_cell_params_t* __restrict__ params)
{
    __shared__ double sh[8];
    const int c = blockIdx.x;
    const BatchCellDev cd = d.cells[c];
    const BatchGridDev gd = d.grids[cd.grid];
    const int off = cd.off, n = cd.n;
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const double* Nc = N + off;
    const double* lc = lam + off;
    double m[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) m[q] = 0.0;
    if (d.kernel >= 0) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double xi = x[i], Ni = Nc[i], li = lc[i];
            vd.h[off + i] = xi * Ni;
            vd.D[off + i] = (i < n - 1) ? (lc[i + 1] - li) / (x[i + 1] - xi) : 0.0;
            const double w[5] = {ia[i], 1.0, a[i], a[i] * a[i], xi};
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                m[q] = fma(w[q], Ni, m[q]);
                m[5 + q] = fma(w[q], li * Ni, m[5 + q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 10; ++q) {
            const double s = block_sum(m[q], sh);
            if (threadIdx.x == 0) vd.mom[c * 16 + q] = s;
        }
    }
    if (d.nq > 0) {
        const pbe_batch_cell_params_t P = params[c];
        const int F = d.selection, ng = gd.n;
        double p0 = 0.0, p1 = 0.0, p2 = 0.0;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const double xj = x[j], Nj = Nc[j];
            const double S = d.Sx ? d.Sx[off + j]
                                  : sel_value_v(F, xj, P.S0, P.v_ref, P.alpha, P.v_min);
            if (!((S != 0.0) && (Nj > kBreakageNMin))) continue;
            double Q = -lc[j];
            for (int q = 0; q < d.nq; ++q) {
                const int e = gd.woff + q * ng + j;
                const int lo = max(d.blo[e], 0);              // clipped below x[0]: lambda_0
                const int hi = min(lo + 1, n - 1);            // its weight is 0 at the cell's end
                Q = fma(d.bwlo[e], lc[lo], Q);
                Q = fma(d.bwhi[e], lc[hi], Q);
            }
            gN[off + j] += S * Q;
            const double NQ = Nj * Q;
            p0 = fma(S / P.S0, NQ, p0);
            if (F == 1) p1 = fma(-(S / P.v_ref), NQ, p1);
            if (F == 2) {
                p1 = fma(-(P.alpha * S / P.v_ref), NQ, p1);
                p2 = fma(S * log(xj / P.v_ref), NQ, p2);
            }
        }
        const double s0 = block_sum(p0, sh);
        const double s1 = block_sum(p1, sh);
        const double s2 = block_sum(p2, sh);
        if (threadIdx.x == 0) {
            gparams[c * 8 + 3] += s0;
            gparams[c * 8 + 4] += s1;
            gparams[c * 8 + 5] += s2;
        }
    }
}

template <int K>
__device__ void batch_vjp_task(const BatchDev& d, const BatchVjpDev& vd, const double* N,
                               const double* lam, double* gN,
                               const pbe_batch_cell_params_t* __restrict__ params, int4 tk,
                               double* red, VjpShared& sm, const TileGroup& G)
{
    const int c = tk.x, I = tk.y;
    const BatchCellDev cd = d.cells[c];
    const BatchGridDev gd = d.grids[cd.grid];
    const int n = cd.n;
    VjpCellView v;
    v.x = d.gx + gd.off;
    v.N = N + cd.off;
    v.h = vd.h + cd.off;
    v.lam = lam + cd.off;
    v.D = vd.D + cd.off;
    v.a = d.ga + gd.off; v.ia = d.gia + gd.off;
    v.Bf = d.gBd + gd.off; v.Sf = d.gSd + gd.off; v.Sl = d.gSl + gd.off; v.Ld = d.gLd + gd.off;
    v.lag0_scale = 2.0;
    v.n = n;
    v.geo = gd.geo != 0;
    // epilogue values through shared memory (no registers held in the loops)
    if (G.lane < 16) {
        const int l = G.lane;
        double val = 0.0;
        if (l < 10) val = vd.mom[c * 16 + l];
        else if (l == 10) val = params[c].beta0;
        else if (l == 11) val = params[c].beta_br;
        else if (l == 12) val = params[c].beta_sh;
        sm.cinfo[G.g][l] = val;
    }
    vjp_tile_accumulate<K>(v, I, 0, n, red, sm, G);    // syncs the group first
    const int tmax = min(VW, n - I);
    if (G.lane < VW) {
        double gB = 0.0, gS = 0.0;
        if (G.lane < tmax) {
            const double* ci = sm.cinfo[G.g];
            double g;
            vjp_tile_row<K>(v, I + G.lane, G.lane, sm.fin[G.g], ci, ci + 5, ci[10], ci[11], ci[12],
                            g, gB, gS);
            gN[cd.off + I + G.lane] += g;
        }
        sm.gsh[G.g][G.lane][0] = gB;
        sm.gsh[G.g][G.lane][1] = gS;
    }
    G.sync();
    if (G.lane == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int t = 0; t < VW; ++t) { s0 += sm.gsh[G.g][t][0]; s1 += sm.gsh[G.g][t][1]; }
        const int slot = vd.tile_off[c] + I / VW;
        vd.tpart[2 * slot + 0] = s0;
        vd.tpart[2 * slot + 1] = s1;
    }
}

template <int K>
__global__ void __launch_bounds__(kMainThreads, 2)
batch_vjp_main_kernel(BatchDev d, BatchVjpDev vd, const double* __restrict__ N,
                      const double* __restrict__ lam, double* __restrict__ gN,
                      const pbe_batch_cell_params_t* __restrict__ params)
{
    extern __shared__ double red[];     // [kVRows][kMainThreads]
    __shared__ VjpShared sm;
    __shared__ int s_b;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_b = atomicAdd(vd.counter, 1);
        __syncthreads();
        const int b = s_b;
        __syncthreads();
        if (b >= vd.n_bundles) break;
        const int4 bu = vd.bundles[b];
        const int T = bu.z;
        const int g = tid / T;
        if (g < bu.y) {
            const TileGroup G{g, tid - g * T, T};
            batch_vjp_task<K>(d, vd, N, lam, gN, params, vd.tasks[bu.x + g], red + g * T, sm, G);
        }
        __syncthreads();
    }
}

// dL/dbeta of each cell: its tiles' partials in tile order.
template <int K>
__global__ void __launch_bounds__(256)
batch_vjp_gfin_kernel(BatchDev d, BatchVjpDev vd, double* __restrict__ gparams)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.n_cells) return;
    double s0 = 0.0, s1 = 0.0;
    for (int t = vd.tile_off[c]; t < vd.tile_off[c + 1]; ++t) {
        s0 += vd.tpart[2 * t];
        s1 += vd.tpart[2 * t + 1];
    }
    if constexpr (K <= 2) gparams[c * 8 + 0] += s0;
    if constexpr (K == 3 || K == 5) gparams[c * 8 + 1] += s0;
    if constexpr (K == 4 || K == 5) gparams[c * 8 + 2] += s1;
}

template <int K>
cudaError_t vjp_k(const BatchDev& d, const BatchVjpDev& vd, const double* N, const double* lam,
                  double* gN, double* gparams, const pbe_batch_cell_params_t* params,
                  cudaStream_t s)
{
    batch_vjp_prep_kernel<<<d.n_cells, 256, 0, s>>>(d, vd, N, lam, gN, gparams, params);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || d.kernel < 0) return e;
    e = cudaMemsetAsync(vd.counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int grid = vd.n_bundles < 2 * d.num_sms ? vd.n_bundles : 2 * d.num_sms;
    if (grid > 0) {
        const size_t smem = sizeof(double) * kVRows * kMainThreads;
        batch_vjp_main_kernel<K><<<grid, kMainThreads, smem, s>>>(d, vd, N, lam, gN, params);
    }
    batch_vjp_gfin_kernel<K><<<(d.n_cells + 255) / 256, 256, 0, s>>>(d, vd, gparams);
    return cudaGetLastError();
}

template <int K>
cudaError_t vjp_attr_k()
{
    return cudaFuncSetAttribute(batch_vjp_main_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(sizeof(double) * kVRows * kMainThreads));
}

// a = w lam' (+ c mu), mu = 0
__global__ void __launch_bounds__(256)
adj_coeff_kernel(double* a, const double* lp, double* mu, double w, double c, long long n,
                 int first)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = first ? w * lp[i] : fma(c, mu[i], w * lp[i]);
    mu[i] = 0.0;
}

__global__ void __launch_bounds__(256) adj_sum_kernel(double* lsum, const double* mu, long long n)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) lsum[i] += mu[i];
}

} // namespace

cudaError_t batch_vjp_setup(int kernel)
{
    switch (kernel < 0 ? 0 : kernel) {
    case 0: return vjp_attr_k<0>();
    case 1: return vjp_attr_k<1>();
    case 2: return vjp_attr_k<2>();
    case 3: return vjp_attr_k<3>();
    case 4: return vjp_attr_k<4>();
    case 5: return vjp_attr_k<5>();
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_vjp(const BatchDev& d, const BatchVjpDev& vd, const double* N, const double* lam,
                      double* gN, double* gparams, const pbe_batch_cell_params_t* params,
                      cudaStream_t s)
{
    switch (d.kernel < 0 ? 0 : d.kernel) {
    case 0: return vjp_k<0>(d, vd, N, lam, gN, gparams, params, s);
    case 1: return vjp_k<1>(d, vd, N, lam, gN, gparams, params, s);
    case 2: return vjp_k<2>(d, vd, N, lam, gN, gparams, params, s);
    case 3: return vjp_k<3>(d, vd, N, lam, gN, gparams, params, s);
    case 4: return vjp_k<4>(d, vd, N, lam, gN, gparams, params, s);
    case 5: return vjp_k<5>(d, vd, N, lam, gN, gparams, params, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_adj_coeff(double* a, const double* lp, double* mu, double w, double c,
                            long long n, bool first, cudaStream_t s)
{
    adj_coeff_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, s>>>(a, lp, mu, w, c, n,
                                                                       first ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t batch_adj_sum(double* lsum, const double* mu, long long n, cudaStream_t s)
{
    adj_sum_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, s>>>(lsum, mu, n);
    return cudaGetLastError();
}

} // namespace pbe_gb300
