// tdse_fft.cu -- batched Fourier interpolation and output spectra for the TDSE.
//
//   mma_tdse_prepare_fields  FourInterp (1DTDSE/sources/tools_fftw3.c:24-68): r2c DFT of the
//                            field, zero padding to k1 N, scale 1/N, c2r DFT.
//   mma_tdse_spectra         calcFFTW3 (tools_fftw3.c:84-143): r2c DFT of a series,
//                            F = dt/sqrt(2 pi) conj(DFT), M2 = dt^2/(2 pi) |DFT|^2,
//                            omega_k = 2 pi k / tmax.
// The DFTs are this library's own (dft.cu: Stockham mixed radix, Bluestein for lengths that are
// not 7-smooth, plans cached per length); the scaling and conjugation are the kernel here.
#include <cuda_runtime.h>

#include "../../include/mma_tdse.h"
#include "dft.cuh"

namespace {

__global__ void spectrum_kernel(const double2* spec, int nc, int n_batch, double c1, double c2, double dxi,
                                double* fsig, long long fsig_stride, double* fm2, long long fm2_stride, double* omega)
{
    const long long total = (long long)nc * n_batch;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(e / nc), k = (int)(e % nc);
        const double2 s = spec[e];
        if (fsig) {
            fsig[b * fsig_stride + 2 * k] = c1 * s.x;
            fsig[b * fsig_stride + 2 * k + 1] = -c1 * s.y;
        }
        if (fm2) fm2[b * fm2_stride + k] = c2 * (s.x * s.x + s.y * s.y);
        if (omega && b == 0) omega[k] = (double)k * dxi;
    }
}

int grid_for(long long total) { return (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096); }

}  // namespace

extern "C" int mma_tdse_prepare_fields(const double* raw, int n_batch, int n_raw, int k1, double* interp,
                                       void* stream)
{
    if (!raw || !interp || n_batch <= 0 || n_raw < 2 || k1 < 1) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (k1 == 1)
        return cudaMemcpyAsync(interp, raw, sizeof(double) * (size_t)n_raw * n_batch, cudaMemcpyDeviceToDevice, st) ==
                       cudaSuccess
                   ? MMA_OK
                   : MMA_ERR_CUDA;
    const int nc = n_raw / 2 + 1, n2 = k1 * n_raw;
    const mma::dft::Plan *pf = nullptr, *pb = nullptr;
    int rc = mma::dft::get_plan(n_raw, st, &pf);
    if (rc == MMA_OK) rc = mma::dft::get_plan(n2, st, &pb);
    if (rc != MMA_OK) return rc;
    double2* spec = nullptr;
    if (cudaMallocAsync((void**)&spec, sizeof(double2) * (size_t)nc * n_batch, st) != cudaSuccess) return MMA_ERR_CUDA;
    rc = mma::dft::r2c(pf, raw, n_raw, spec, nc, n_batch, st);
    // the spectrum zero-padded to k1 N / 2 + 1 bins and scaled by 1/N, then the inverse transform
    if (rc == MMA_OK) rc = mma::dft::c2r(pb, spec, nc, nc, interp, n2, n_batch, 1.0 / n_raw, st);
    cudaFreeAsync(spec, st);
    if (rc == MMA_OK && cudaGetLastError() != cudaSuccess) rc = MMA_ERR_CUDA;
    return rc;
}

extern "C" int mma_tdse_spectra(const double* series, int64_t series_stride, int n_batch, int n_out, double dt,
                                double tmax, double* fsig, int64_t fsig_stride, double* fm2, int64_t fm2_stride,
                                double* omega, void* stream)
{
    if (!series || n_batch <= 0 || n_out < 2 || series_stride < n_out || !(tmax > 0.0)) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int nc = n_out / 2 + 1;
    const mma::dft::Plan* pf = nullptr;
    int rc = mma::dft::get_plan(n_out, st, &pf);
    if (rc != MMA_OK) return rc;
    double2* spec = nullptr;
    if (cudaMallocAsync((void**)&spec, sizeof(double2) * (size_t)nc * n_batch, st) != cudaSuccess) return MMA_ERR_CUDA;
    rc = mma::dft::r2c(pf, series, series_stride, spec, nc, n_batch, st);
    if (rc == MMA_OK) {
        const double two_pi = 6.283185307179586476925286766559;
        spectrum_kernel<<<grid_for((long long)nc * n_batch), 256, 0, st>>>(
            spec, nc, n_batch, dt / sqrt(two_pi), dt * dt / two_pi, two_pi / tmax, fsig, fsig_stride, fm2,
            fm2_stride, omega);
    }
    cudaFreeAsync(spec, st);
    if (rc == MMA_OK && cudaGetLastError() != cudaSuccess) rc = MMA_ERR_CUDA;
    return rc;
}
