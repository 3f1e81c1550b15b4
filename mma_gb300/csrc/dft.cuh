// dft.cuh -- this library's batched real DFTs in FP64 (FFTW's conventions, which the reference's
// tools_fftw3.c uses):
//   r2c  X_k = sum_j x_j exp(-2 pi i j k / n),  k = 0 .. n/2
//   c2r  x_j = scale * sum_{k=0}^{n-1} X_k exp(+2 pi i j k / n),  X_{n-k} = conj(X_k)
//        (the imaginary parts of the DC bin and, for even n, of the Nyquist bin are ignored)
// An even-length row is transformed as a complex row of half the length (real packing); the
// complex DFT of length L is a Stockham mixed-radix FFT (radices 8, 4, 2, 7, 5, 3) when L is
// 7-smooth, and Bluestein's chirp convolution over the smallest 7-smooth M >= 2L - 1 otherwise.
// Rows whose FFT length fits in shared memory run one CTA per row, every pass in shared memory;
// longer rows run one launch per pass through global memory.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace mma {
namespace dft {

struct Plan;

// The plan of a real DFT of length n on the current device, created and cached on first use
// (device tables, and the CTA size picked by timing the candidates).  Plan creation allocates
// device memory and synchronises, so it is refused (MMA_ERR_DFT) while `st` is being captured:
// make the first call for each length outside stream capture.
int get_plan(int n, cudaStream_t st, const Plan** out);

// r2c of n_batch rows: row b of x at x + b x_stride (n doubles), of X at X + b X_stride
// (n/2 + 1 complex values).
int r2c(const Plan* p, const double* x, int64_t x_stride, double2* X, int64_t X_stride, int n_batch,
        cudaStream_t st);

// c2r of n_batch rows from the first n_bins bins of each X row (bins n_bins .. n/2 are zero),
// times `scale`.  The global-memory path (FFT length above 7168) takes its two work buffers
// from the stream-ordered allocator.
int c2r(const Plan* p, const double2* X, int64_t X_stride, int n_bins, double* x, int64_t x_stride, int n_batch,
        double scale, cudaStream_t st);

}  // namespace dft
}  // namespace mma
