// tdse_solver.cuh -- CTA-wide tridiagonal solve with a precomputed factorisation.
//
// The reference solves every Crank-Nicolson step and every inverse-iteration
// step with a serial Thomas sweep (1DTDSE/sources/tridiag.c:26-70), refactoring
// a matrix that never changes.  Here the factorisation is computed once per grid
// and the solve is split over the kMThreads threads of a CTA:
//
//   forward    y_j = ib_j r_j - h_j y_{j-1}          ib = 1/beta, h_j = a_j/beta_j
//   backward   u_j = y_j - g_j u_{j+1}               g_j = c_j/beta_j
//
// Thread t owns the contiguous chunk j in [t m, t m + m).  It runs both sweeps
// locally from zero boundary values, and the exact solution follows from
//   y_j = yl_j + F_j Y_{t-1},  F_j = prod_{k=chunk start}^{j} (-h_k)
//   u_j = ul_j + G_j U_{t+1},  G_j = prod_{k=j}^{chunk end} (-g_k)
// where the chunk-boundary values Y (last y of each chunk) and U (first u of each
// chunk) come from a CTA-wide scan of the affine maps Y_t = yl_end + F_end Y_{t-1}
// (forward) and U_t = ul_start + G_start U_{t+1} (backward): warp shuffles, then
// the eight warp totals through shared memory.  The work stays O(n) and the
// result equals Thomas up to rounding.
//
// Storage is "chunk-interleaved": site j = t m + i lives at index q = i T + t, so a
// warp touching element i of its 32 chunks reads 32 consecutive entries.
#pragma once

#include "common.cuh"

namespace mma {

__device__ __forceinline__ double axpy_(double c, double y, double b) { return fma(c, y, b); }
__device__ __forceinline__ cd axpy_(cd c, cd y, cd b) { return cfma(c, y, b); }
__device__ __forceinline__ double mul_(double a, double b) { return a * b; }
__device__ __forceinline__ cd mul_(cd a, cd b) { return cmul(a, b); }
__device__ __forceinline__ double zero_(double) { return 0.0; }
__device__ __forceinline__ cd zero_(cd) { return cd{0.0, 0.0}; }
__device__ __forceinline__ double shup_(double v, int d) { return shfl_up(v, d); }
__device__ __forceinline__ cd shup_(cd v, int d) { return cd{shfl_up(v.re, d), shfl_up(v.im, d)}; }
__device__ __forceinline__ double shdn_(double v, int d) { return shfl_down(v, d); }
__device__ __forceinline__ cd shdn_(cd v, int d) { return cd{shfl_down(v.re, d), shfl_down(v.im, d)}; }

// Exclusive forward scan of Y_t = b_t + c_t Y_{t-1} (Y_{-1} = 0): returns Y_{t-1}.
// sc/sb: kWarps entries of shared scratch.  Contains one __syncthreads.
template <typename T>
__device__ __forceinline__ T scan_forward(T c, T b, T* sc, T* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T cp = shup_(c, d), bp = shup_(b, d);
        if (lane >= d) {
            b = axpy_(c, bp, b);
            c = mul_(c, cp);
        }
    }
    if (lane == 31) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    T yw = zero_(b);
    for (int q = 0; q < w; q++) yw = axpy_(sc[q], yw, sb[q]);
    T cp = shup_(c, 1), bp = shup_(b, 1);
    return lane == 0 ? yw : axpy_(cp, yw, bp);
}

// Exclusive backward scan of U_t = b_t + c_t U_{t+1} (U_T = 0): returns U_{t+1}.
template <typename T>
__device__ __forceinline__ T scan_backward(T c, T b, T* sc, T* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T cp = shdn_(c, d), bp = shdn_(b, d);
        if (lane + d < 32) {
            b = axpy_(c, bp, b);
            c = mul_(c, cp);
        }
    }
    if (lane == 0) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    T uw = zero_(b);
    for (int q = kWarps - 1; q > w; q--) uw = axpy_(sc[q], uw, sb[q]);
    T cp = shdn_(c, 1), bp = shdn_(b, 1);
    return lane == 31 ? uw : axpy_(cp, uw, bp);
}

}  // namespace mma
