// =============================================================================
// peak_probe.cu -- FP64 throughput probes (libpbe_probe.so), used by bench.py
// as roofline denominators:
//  * pbe_probe_dfma_tflops: 8 CTAs per SM, 8 independent DFMA chains per
//    thread (2 flops per DFMA) -- the FP64 CUDA-core pipe of the pair kernels;
//  * pbe_probe_dmma_tflops: 8 CTAs per SM, 8 independent mma.sync m8n8k4 f64
//    accumulators per warp (512 flops per warp instruction) -- the FP64
//    tensor pipe of the death GEMM.
// The best of `reps` CUDA-event-timed launches is returned, in TFLOP/s.
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
__global__ void __launch_bounds__(256) dmma_chains(double* out, int iters, double a, double b)
{
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) { c[k][0] = threadIdx.x + k; c[k][1] = c[k][0] + 0.5; }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                         : "+d"(c[k][0]), "+d"(c[k][1]) : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

using Launcher = void (*)(int blocks, int threads, double* out, int iters, cudaStream_t s);

void launch_dfma(int blocks, int threads, double* out, int iters, cudaStream_t s)
{
    dfma_chains<<<blocks, threads, 0, s>>>(out, iters, 1.0000001, 1e-9);
}

void launch_dmma(int blocks, int threads, double* out, int iters, cudaStream_t s)
{
    dmma_chains<<<blocks, threads, 0, s>>>(out, iters, 1e-3, 1e-3);
}

// flops_per_iter_thread: flops one thread contributes per loop iteration
double probe(Launcher launch, double flops_per_iter_thread, int iters, int reps, void* stream)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int blocks = sms * 8, threads = 256;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* out = nullptr;
    if (cudaMallocAsync(&out, sizeof(double) * blocks * threads, s) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch(blocks, threads, out, 50, s);
    double best = 0.0;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, s);
        launch(blocks, threads, out, iters, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = flops_per_iter_thread * iters * static_cast<double>(blocks) * threads
                        / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    cudaStreamSynchronize(s);
    return cudaGetLastError() == cudaSuccess ? best : -1.0;
}
} // namespace

extern "C" double pbe_probe_dmma_tflops(int reps, void* stream)
{
    // 8 mma per iteration per warp, 512 flops each, spread over 32 threads
    return probe(launch_dmma, 8.0 * 512.0 / 32.0, 2000, reps, stream);
}

extern "C" double pbe_probe_dfma_tflops(int reps, void* stream)
{
    return probe(launch_dfma, 2.0 * 8.0, 4000, reps, stream);
}
