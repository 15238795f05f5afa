// =============================================================================
// death_gemm.cu -- aggregation death term of batched cells, two ways
// (no counterpart in the reference, whose pair kernel deposits -rate at j and
// k pair by pair: src/aggregation_kernels.cuh:213-221).
//
//   death[c, i] = N[c, i] * D[c, i],   D[c, i] = sum_k beta_c(x_i, x_k) N[c, k]
//
// MOMENTS (the form the RHS kernels use): beta splits into at most five
// separable terms in x_k^p (p = -1/3, 0, 1/3, 2/3, 1), so D is a combination
// of five per-cell moments -- O(n) per cell on the CUDA cores.
//
// DMMA: for the cells sharing a grid, D = A B^T is a GEMM with
// A[c, k] = coef_s(c) N[c, k] and B[i, k] = f_s(x_i, x_k) per separable
// component s (Brownian a_i/a_k + a_k/a_i + 2, shear (a_i + a_k)^3, or
// 1, x_i + x_k, x_i x_k), the components concatenated along k so one GEMM
// covers Brownian + shear with per-cell coefficients. It runs on the FP64
// tensor cores with mma.sync.m8n8k4.f64 (tcgen05 has no FP64 kind); B tiles
// are generated in shared memory from the grid's cube roots, never stored.
// A CTA owns 64 cells x 64 bins (4 warps of 32 x 32) and one of S slices of
// the k range (grid y): with few cells per grid there are few 64 x 64 tiles,
// so the slices give the SMs enough CTAs; each slice stores its partial D and
// death_reduce_kernel adds the S partials in slice order and multiplies by N
// (S = 1: the CTA writes N D itself). 2 n^2 C flops per component. On GB300 the FP64 MMA rate is no higher than the DFMA rate, so
// this form is measured beside the moment form rather than used by the RHS.
// =============================================================================
#include "batch_internal.cuh"
#include "agg_tile.cuh"

namespace pbe_gb300 {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16, kPad = 8;

__device__ __forceinline__ void mma884(double& c0, double& c1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
}

template <int K> struct Comps { static constexpr int n = (K == 5) ? 2 : 1; };

// f_s(x_i, x_k) of component s (beta without its coefficient)
template <int K>
__device__ __forceinline__ double comp_value(int s, double xi, double ai, double iai, double xk,
                                             double ak, double iak)
{
    if constexpr (K == 0) return 1.0;
    else if constexpr (K == 1) return xi + xk;
    else if constexpr (K == 2) return xi * xk;
    else {
        const bool brown = (K == 3) || (K == 5 && s == 0);
        if (brown) return fma(ai, iak, ak * iai) + 2.0;
        const double t = ai + ak;
        return (t * t) * t;
    }
}

template <int K>
__device__ __forceinline__ double comp_coef(int s, const pbe_batch_cell_params_t& P)
{
    if constexpr (K <= 2) return P.beta0;
    else if constexpr (K == 3) return P.beta_br;
    else if constexpr (K == 4) return P.beta_sh;
    else return s == 0 ? P.beta_br : P.beta_sh;
}

// B of every grid, once per plan: Bm[boff[g] + i * (NC ld) + s ld + k] =
// f_s(x_i, x_k), ld = n_g rounded up to kBK (grid-stride over the grid's
// n_g x NC ld entries; the padding is 0).
template <int K>
__global__ void __launch_bounds__(256)
death_b_kernel(BatchDev d, int g, double* __restrict__ Bm)
{
    constexpr int NC = Comps<K>::n;
    const BatchGridDev gd = d.grids[g];
    const int n = gd.n, ld = (n + kBK - 1) / kBK * kBK;
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const long long cols = static_cast<long long>(NC) * ld, total = cols * n;
    for (long long e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
        const int i = static_cast<int>(e / cols);
        const int c = static_cast<int>(e - static_cast<long long>(i) * cols);
        const int s = c / ld, k = c - s * ld;
        Bm[e] = (k < n) ? comp_value<K>(s, x[i], a[i], ia[i], x[k], a[k], ia[k]) : 0.0;
    }
}

// item = {grid, first row in gcells, rows (<= 64), first bin}; k slice
// blockIdx.y of gridDim.y; part: [gridDim.y][total] partial D (null when
// gridDim.y == 1: out = N D directly).
template <int K>
__global__ void __launch_bounds__(128)
death_dmma_kernel(BatchDev d, const double* __restrict__ N,
                  const pbe_batch_cell_params_t* __restrict__ params, double* __restrict__ out,
                  const int4* __restrict__ items, const int* __restrict__ gcells,
                  double* __restrict__ part, long long total, const double* __restrict__ Bm,
                  const long long* __restrict__ boff)
{
    __shared__ double As[kBK][kBM + kPad];
    __shared__ double Bs[kBK][kBN + kPad];
    __shared__ int s_off[kBM], s_n[kBM];
    __shared__ double s_coef[Comps<K>::n][kBM];
    __shared__ int s_kmax;
    constexpr int NC = Comps<K>::n;
    const int4 it = items[blockIdx.x];
    const BatchGridDev gd = d.grids[it.x];
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const int rows = it.z, i0 = it.w;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int wm = warp >> 1, wn = warp & 1;
    if (tid == 0) s_kmax = 0;
    __syncthreads();
    if (tid < kBM) {
        int off = 0, n = 0;
        pbe_batch_cell_params_t P{};
        if (tid < rows) {
            const int c = gcells[it.y + tid];
            const BatchCellDev cd = d.cells[c];
            off = cd.off; n = cd.n; P = params[c];
        }
        s_off[tid] = off;
        s_n[tid] = n;
        for (int s = 0; s < NC; ++s) s_coef[s][tid] = comp_coef<K>(s, P);
        atomicMax(&s_kmax, n);
    }
    __syncthreads();
    const int kmax = s_kmax;
    double acc[4][4][2];
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) acc[mi][ni][0] = acc[mi][ni][1] = 0.0;

    // components concatenated along k with a stride of kmax rounded up to kBK,
    // so a k block lies in one component (the padding has A = 0)
    const int kpad = (kmax + kBK - 1) / kBK * kBK;
    const int ldg = (gd.n + kBK - 1) / kBK * kBK;                 // B's component stride
    const double* Bg = Bm + boff[it.x];
    const int ktot = NC * kpad;
    const int S = gridDim.y;
    const int kc = ((ktot + S - 1) / S + kBK - 1) / kBK * kBK;     // slice length, kBK multiple
    const int kbeg = min(ktot, static_cast<int>(blockIdx.y) * kc);
    const int kend = min(ktot, kbeg + kc);
    for (int kb = kbeg; kb < kend; kb += kBK) {
        const int sc = kb / kpad, kb0 = kb - sc * kpad;     // component, its first k here
        // A tile: rows = cells, k contiguous in N (coalesced)
        for (int e = tid; e < kBM * kBK; e += blockDim.x) {
            const int m = e / kBK, kk = e - m * kBK;
            const int k = kb0 + kk;
            double v = 0.0;
            if (kb + kk < kend && k < s_n[m]) v = s_coef[sc][m] * N[s_off[m] + k];
            As[kk][m] = v;
        }
        // B tile: the grid's precomputed B (16 consecutive k per bin)
        for (int e = tid; e < kBN * kBK; e += blockDim.x) {
            const int ib = e / kBK, kk = e - ib * kBK;
            const int k = kb0 + kk, bin = i0 + ib;
            double v = 0.0;
            if (kb + kk < kend && k < kmax && bin < gd.n)
                v = Bg[static_cast<size_t>(bin) * (NC * ldg) + sc * ldg + k];
            Bs[kk][ib] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 4) {
            double af[4], bf[4];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi) af[mi] = As[kk + t][wm * 32 + mi * 8 + g];
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) bf[ni] = Bs[kk + t][wn * 32 + ni * 8 + g];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) mma884(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) {
        const int m = wm * 32 + mi * 8 + g;
        if (m >= rows) continue;
        const int off = s_off[m], n = s_n[m];
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int bin = i0 + wn * 32 + ni * 8 + 2 * t + r;
                if (bin >= n) continue;
                if (part) part[blockIdx.y * total + off + bin] = acc[mi][ni][r];
                else out[off + bin] = N[off + bin] * acc[mi][ni][r];
            }
    }
}

// out = N (sum of the S slices' partial D, in slice order), every packed bin.
__global__ void __launch_bounds__(256)
death_reduce_kernel(const double* __restrict__ N, const double* __restrict__ part, int S,
                    long long total, double* __restrict__ out)
{
    for (long long e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
        double s_ = 0.0;
        for (int q = 0; q < S; ++q) s_ += part[q * total + e];
        out[e] = N[e] * s_;
    }
}

// Moment form: one CTA per cell.
template <int K>
__global__ void __launch_bounds__(256)
death_moments_kernel(BatchDev d, const double* __restrict__ N,
                     const pbe_batch_cell_params_t* __restrict__ params, double* __restrict__ out)
{
    __shared__ double sh[8];
    const BatchCellDev cd = d.cells[blockIdx.x];
    const BatchGridDev gd = d.grids[cd.grid];
    const pbe_batch_cell_params_t P = params[blockIdx.x];
    const double* x = d.gx + gd.off;
    const double* a = d.ga + gd.off;
    const double* ia = d.gia + gd.off;
    const double* Nc = N + cd.off;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < cd.n; i += blockDim.x) {
        const double y = Nc[i];
        m[0] = fma(ia[i], y, m[0]);
        m[1] += y;
        m[2] = fma(a[i], y, m[2]);
        m[3] = fma(a[i] * a[i], y, m[3]);
        m[4] = fma(x[i], y, m[4]);
    }
    double M[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) M[q] = block_sum(m[q], sh);
    for (int i = threadIdx.x; i < cd.n; i += blockDim.x)
        out[cd.off + i] = Nc[i] * death_factor<K>(x[i], a[i], ia[i], M, P.beta0, P.beta_br, P.beta_sh);
}

template <int K>
cudaError_t death_b_k(const BatchDev& d, const int* grids_used, int n_used, double* Bm,
                      const long long* hboff, cudaStream_t s)
{
    for (int q = 0; q < n_used; ++q) {
        const int g = grids_used[q];
        death_b_kernel<K><<<16 * (d.num_sms > 0 ? d.num_sms : 1), 256, 0, s>>>(d, g, Bm + hboff[g]);
    }
    return cudaGetLastError();
}

template <int K>
cudaError_t death_k(const BatchDev& d, const double* N, const pbe_batch_cell_params_t* params,
                    double* out, int method, const int4* items, int n_items, const int* gcells,
                    double* part, int S, long long total, const double* Bm, const long long* boff,
                    cudaStream_t s)
{
    if (method == 0) {
        death_moments_kernel<K><<<d.n_cells, 256, 0, s>>>(d, N, params, out);
    } else {
        if (n_items <= 0) return cudaSuccess;
        const bool split = S > 1 && part;
        death_dmma_kernel<K><<<dim3(n_items, split ? S : 1), 128, 0, s>>>(
            d, N, params, out, items, gcells, split ? part : nullptr, total, Bm, boff);
        if (split) {
            const long long b = (total + 255) / 256, cap = 16LL * (d.num_sms > 0 ? d.num_sms : 1);
            death_reduce_kernel<<<static_cast<int>(b < cap ? b : cap), 256, 0, s>>>(N, part, S,
                                                                                     total, out);
        }
    }
    return cudaGetLastError();
}

} // namespace

cudaError_t batch_death_b(const BatchDev& d, const int* grids_used, int n_used, double* Bm,
                          const long long* hboff, cudaStream_t s)
{
    switch (d.kernel) {
    case 0: return death_b_k<0>(d, grids_used, n_used, Bm, hboff, s);
    case 1: return death_b_k<1>(d, grids_used, n_used, Bm, hboff, s);
    case 2: return death_b_k<2>(d, grids_used, n_used, Bm, hboff, s);
    case 3: return death_b_k<3>(d, grids_used, n_used, Bm, hboff, s);
    case 4: return death_b_k<4>(d, grids_used, n_used, Bm, hboff, s);
    case 5: return death_b_k<5>(d, grids_used, n_used, Bm, hboff, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t batch_death(const BatchDev& d, const double* N, const pbe_batch_cell_params_t* params,
                        double* out, int method, const int4* items, int n_items,
                        const int* gcells, double* part, int S, long long total, const double* Bm,
                        const long long* boff, cudaStream_t s)
{
    switch (d.kernel) {
    case 0: return death_k<0>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    case 1: return death_k<1>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    case 2: return death_k<2>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    case 3: return death_k<3>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    case 4: return death_k<4>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    case 5: return death_k<5>(d, N, params, out, method, items, n_items, gcells, part, S, total, Bm, boff, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace pbe_gb300
