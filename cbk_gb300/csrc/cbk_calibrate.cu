// cbk_calibrate.cu -- measured FP64 / FP32 fused multiply-add rates of the
// current device, the denominators of the FP64-pipe roofline the solves are
// bound by on a GB300 (its FP64 rate is ~1/58 of FP32). Each thread runs
// eight independent FMA chains; the launch fills every SM several times over.
#include "../../include/cbk_cuda.h"

#include <cuda_runtime.h>

namespace {

template <typename T> __global__ void k_fma_chains(T *out, int iters, T a, T b)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    T x0 = T(tid) * T(1e-9), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    out[tid] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T> int rate(int iters, double *tflops)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    const int threads = 256, blocks = sms * 8, n = threads * blocks;
    T *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(T) * n) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        k_fma_chains<T><<<blocks, threads>>>(buf, iters, T(1.0000001), T(1e-7));
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (err != cudaSuccess) return CBK_CUDA_ERROR_BASE + (int)err;
    *tflops = 2.0 * 8.0 * iters * (double)n / (best * 1e-3) / 1e12;
    return 0;
}

} // namespace

extern "C" int cbk_cuda_measure_fma_rate(int fp64, double *tflops)
{
    return fp64 ? rate<double>(2048, tflops) : rate<float>(65536, tflops);
}
