// peaks.cu -- CUDA-core FMA throughput microbenchmarks (diagnostic entry point).
//
// The roofline denominators for the FP64 and FP32 (CUDA-core) kernels of this engine
// are not among the measured peaks (HBM copy, cuBLAS bf16), so they are
// measured here: a grid of 152 * 8 CTAs, each thread running independent FMA chains
// (8-way instruction-level parallelism) for a fixed number of iterations, timed with
// CUDA events on a private stream.
#include <cuda_runtime.h>

#include "../../include/cqpi.h"

namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_loop(T *out, int iters, T a, T b)
{
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-12345.678) out[blockIdx.x] = s;   // keeps the chains alive
}

template <class T>
int run(double *tflops, int iters)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CQPI_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    cudaStream_t s;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&out, sizeof(T) * blocks) != cudaSuccess) return CQPI_ERR_ALLOC;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_loop<T><<<blocks, threads, 0, s>>>(out, iters / 8, (T)0.999999, (T)1e-7);   // warm-up
    cudaEventRecord(e0, s);
    fma_loop<T><<<blocks, threads, 0, s>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1, s);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    if (err != cudaSuccess) return CQPI_ERR_CUDA;
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return CQPI_OK;
}

}  // namespace

extern "C" int cqpi_measure_fma_peak(int32_t kind, double *tflops)
{
    if (!tflops) return CQPI_ERR_ARG;
    if (kind == 0) return run<double>(tflops, 256);
    if (kind == 1) return run<float>(tflops, 4096);
    return CQPI_ERR_ARG;
}
