// probe.cu -- FMA-rate probe used as the roofline denominator of FP64/FP32-bound kernels.
#include <cuda_runtime.h>

#include "../../include/mma_diag.h"

namespace {

constexpr int kIlp = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_loop(T* out, int iters, T a, T b)
{
    T x[kIlp];
#pragma unroll
    for (int i = 0; i < kIlp; i++) x[i] = (T)(threadIdx.x * 1e-3 + i);
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < kIlp; i++) x[i] = fma(x[i], a, b);
    T s = 0;
#pragma unroll
    for (int i = 0; i < kIlp; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int run(int iters, double* rate)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 6;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 4, threads = 256;
    T* out = nullptr;
    if (cudaMalloc((void**)&out, sizeof(T) * blocks * threads) != cudaSuccess) return 3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_loop<T><<<blocks, threads>>>(out, 16, (T)1.0000001, (T)1e-9);
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        fma_loop<T><<<blocks, threads>>>(out, iters, (T)1.0000001, (T)1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return 3;
    *rate = 2.0 * kIlp * (double)iters * blocks * threads / (best * 1e-3);
    return 0;
}

}  // namespace

extern "C" int mma_probe_fma_peak(int precision, double* flops_per_s)
{
    if (!flops_per_s) return 1;
    return precision == 0 ? run<double>(2000, flops_per_s) : run<float>(20000, flops_per_s);
}
