// common.cuh -- small device helpers shared by the TDSE and Hankel kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mma {

constexpr int kThreads = 256;  // CTA size of every TDSE kernel (tables are laid out for it)
constexpr int kWarps = kThreads / 32;

// ---------------------------------------------------------------- complex FP64
struct cd {
    double re, im;
};
__device__ __forceinline__ cd mk(double r, double i) { return cd{r, i}; }
__device__ __forceinline__ cd operator+(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd operator-(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cd cmul(cd a, cd b) { return cd{fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re)}; }
// a + b*c
__device__ __forceinline__ cd cfma(cd b, cd c, cd a)
{
    return cd{fma(b.re, c.re, fma(-b.im, c.im, a.re)), fma(b.re, c.im, fma(b.im, c.re, a.im))};
}
// a - b*c
__device__ __forceinline__ cd cfms(cd b, cd c, cd a)
{
    return cd{fma(-b.re, c.re, fma(b.im, c.im, a.re)), fma(-b.re, c.im, fma(-b.im, c.re, a.im))};
}
__device__ __forceinline__ cd cdiv(cd a, cd b)
{
    double d = b.re * b.re + b.im * b.im;
    return cd{(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__device__ __forceinline__ cd ld2(const double* p) { double2 v = *reinterpret_cast<const double2*>(p); return cd{v.x, v.y}; }
__device__ __forceinline__ void st2(double* p, cd v) { *reinterpret_cast<double2*>(p) = make_double2(v.re, v.im); }

__device__ __forceinline__ double shfl_up(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_down(double v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_xor(double v, int d) { return __shfl_xor_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_idx(double v, int l) { return __shfl_sync(0xffffffffu, v, l); }

// Sum of NV doubles over the CTA.  Every thread gets the totals; the order of the
// additions is fixed, so the result is reproducible.  `red` holds NW*NV doubles (NW warps).
template <int NV, int NW = kWarps>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red)
{
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) v[k] += shfl_xor(v[k], d);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) red[w * NV + k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NW; q++) s += red[q * NV + k];
        v[k] = s;
    }
    __syncthreads();
}

}  // namespace mma
