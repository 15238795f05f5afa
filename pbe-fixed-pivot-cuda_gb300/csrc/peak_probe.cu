// =============================================================================
// peak_probe.cu -- FP64 pipe throughput probe (libpbe_probe.so), used by
// bench.py as the roofline denominator for the FP64-bound pair kernel.
// A grid of 8 CTAs per SM runs 8 independent DFMA chains per thread; the best
// of `reps` CUDA-event-timed launches gives TFLOP/s (2 flops per DFMA).
// =============================================================================
#include <cuda_runtime.h>

namespace {
__global__ void __launch_bounds__(256) dfma_chains(double* out, int iters, double b, double c)
{
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}
} // namespace

extern "C" double pbe_probe_dfma_tflops(int reps, void* stream)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int blocks = sms * 8, threads = 256, iters = 4000;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* out = nullptr;
    if (cudaMallocAsync(&out, sizeof(double) * blocks * threads, s) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_chains<<<blocks, threads, 0, s>>>(out, 50, 1.0000001, 1e-9);
    double best = 0.0;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, s);
        dfma_chains<<<blocks, threads, 0, s>>>(out, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess ? best : -1.0;
}
