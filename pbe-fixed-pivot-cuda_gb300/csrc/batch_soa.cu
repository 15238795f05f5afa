// =============================================================================
// batch_soa.cu -- mesh-field (structure-of-arrays) layout <-> the plan's packed
// cell layout, for coupling the batched integrators to a CFD solver.
//
// A CFD code keeps one field per PBE bin over its mesh cells: soa[i * ld + c]
// is bin i of mesh cell c (ld >= n_cells). The plan packs cell c's bins
// contiguously at N[off_c .. off_c + n_c). Both directions are one tiled
// transpose: a 32 x 32 tile (cells x bins) is read coalesced along the cells,
// staged in shared memory (padded against bank conflicts) and written
// coalesced along the bins; bins at or beyond a cell's n_c are not touched.
// =============================================================================
#include "batch_internal.cuh"

namespace pbe_gb300 {
namespace {

constexpr int kTile = 32;

// to_packed: N[off_c + i] = soa[i ld + c]; else soa[i ld + c] = N[off_c + i].
template <bool TO_PACKED>
__global__ void __launch_bounds__(kTile * 8)
soa_kernel(BatchDev d, const double* __restrict__ src, double* __restrict__ dst, long long ld,
           int max_n)
{
    __shared__ double tile[kTile][kTile + 1];
    const int c0 = blockIdx.x * kTile, i0 = blockIdx.y * kTile;
    const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;   // 32 x 8 threads
    if (i0 >= max_n) return;
    if (TO_PACKED) {
        // read rows of bins (coalesced over cells)
        for (int r = ty; r < kTile; r += 8) {
            const int i = i0 + r, c = c0 + tx;
            double v = 0.0;
            if (c < d.n_cells && i < d.cells[c].n) v = src[static_cast<long long>(i) * ld + c];
            tile[r][tx] = v;
        }
        __syncthreads();
        // write each cell's bins (coalesced over bins)
        for (int r = ty; r < kTile; r += 8) {
            const int c = c0 + r, i = i0 + tx;
            if (c < d.n_cells) {
                const BatchCellDev cd = d.cells[c];
                if (i < cd.n) dst[cd.off + i] = tile[tx][r];
            }
        }
    } else {
        for (int r = ty; r < kTile; r += 8) {
            const int c = c0 + r, i = i0 + tx;
            double v = 0.0;
            if (c < d.n_cells) {
                const BatchCellDev cd = d.cells[c];
                if (i < cd.n) v = src[cd.off + i];
            }
            tile[tx][r] = v;
        }
        __syncthreads();
        for (int r = ty; r < kTile; r += 8) {
            const int i = i0 + r, c = c0 + tx;
            if (c < d.n_cells && i < d.cells[c].n) dst[static_cast<long long>(i) * ld + c] = tile[r][tx];
        }
    }
}

} // namespace

cudaError_t batch_soa(const BatchDev& d, const double* src, double* dst, long long ld, int max_n,
                      bool to_packed, cudaStream_t s)
{
    if (d.n_cells <= 0 || max_n <= 0) return cudaSuccess;
    const dim3 grid((d.n_cells + kTile - 1) / kTile, (max_n + kTile - 1) / kTile);
    if (grid.y > 65535u) return cudaErrorInvalidValue;
    if (to_packed) soa_kernel<true><<<grid, kTile * 8, 0, s>>>(d, src, dst, ld, max_n);
    else soa_kernel<false><<<grid, kTile * 8, 0, s>>>(d, src, dst, ld, max_n);
    return cudaGetLastError();
}

} // namespace pbe_gb300
