// tdse_fft.cu -- batched Fourier interpolation and output spectra for the TDSE.
//
//   mma_tdse_prepare_fields  FourInterp (1DTDSE/sources/tools_fftw3.c:24-68): r2c DFT of the
//                            field, zero padding to k1 N, scale 1/N, c2r DFT.
//   mma_tdse_spectra         calcFFTW3 (tools_fftw3.c:84-143): r2c DFT of a series,
//                            F = dt/sqrt(2 pi) conj(DFT), M2 = dt^2/(2 pi) |DFT|^2,
//                            omega_k = 2 pi k / tmax.
// The DFTs are cuFFT double-precision transforms (batched, plans cached per shape);
// the scaling, padding and conjugation are kernels here.
#include <cuda_runtime.h>
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>

#include "../../include/mma_tdse.h"

namespace {

std::mutex g_plan_mu;
std::map<std::tuple<int, int, int, long long, long long, int>, cufftHandle> g_plans;

// Plan cache keyed by (device, type, n, idist, odist, batch).
int get_plan(cufftType type, int n, long long idist, long long odist, int batch, cufftHandle* out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MMA_ERR_NO_DEVICE;
    auto key = std::make_tuple(dev * 16 + (int)type, n, idist, odist, batch, 0);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        *out = it->second;
        return MMA_OK;
    }
    cufftHandle p;
    int nn[1] = {n};
    int inembed[1] = {(int)idist}, onembed[1] = {(int)odist};
    if (cufftPlanMany(&p, 1, nn, inembed, 1, (int)idist, onembed, 1, (int)odist, type, batch) != CUFFT_SUCCESS)
        return MMA_ERR_CUFFT;
    g_plans[key] = p;
    *out = p;
    return MMA_OK;
}

__global__ void pad_scale_kernel(const double2* spec, int nc, double2* pad, int nc2, int n_batch, double inv_n)
{
    const long long total = (long long)nc2 * n_batch;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(e / nc2), k = (int)(e % nc2);
        double2 v = make_double2(0.0, 0.0);
        if (k < nc) {
            double2 s = spec[(long long)b * nc + k];
            v = make_double2(s.x * inv_n, s.y * inv_n);
        }
        pad[e] = v;
    }
}

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

__global__ void gather_rows_kernel(const double* src, long long src_stride, int n, double* dst, long long dst_stride,
                                   int n_batch)
{
    const long long total = (long long)dst_stride * n_batch;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long b = e / dst_stride, k = e % dst_stride;
        dst[e] = (k < n) ? src[b * src_stride + k] : 0.0;
    }
}

int grid_for(long long total) { return (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096); }

}  // namespace

// the plan cache, for the other FFT users of the library (tdse_analysis.cu)
int mma_fft_get_plan_d2z(int n, long long idist, long long odist, int batch, cufftHandle* out)
{
    return get_plan(CUFFT_D2Z, n, idist, odist, batch, out);
}

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
    const int nc = n_raw / 2 + 1, n2 = k1 * n_raw, nc2 = n2 / 2 + 1;
    // rows handed to cuFFT use even strides so every row is aligned to its complex type
    const long long ri = (n_raw + 1) / 2 * 2, ro = (n2 + 1) / 2 * 2;
    double2 *spec = nullptr, *pad = nullptr;
    double *rin = nullptr, *rout = nullptr;
    int rc = MMA_OK;
    if (cudaMallocAsync((void**)&spec, sizeof(double2) * (size_t)nc * n_batch, st) != cudaSuccess ||
        cudaMallocAsync((void**)&pad, sizeof(double2) * (size_t)nc2 * n_batch, st) != cudaSuccess ||
        cudaMallocAsync((void**)&rin, sizeof(double) * (size_t)ri * n_batch, st) != cudaSuccess ||
        cudaMallocAsync((void**)&rout, sizeof(double) * (size_t)ro * n_batch, st) != cudaSuccess)
        rc = MMA_ERR_CUDA;
    cufftHandle pf, pb;
    if (rc == MMA_OK && (rc = get_plan(CUFFT_D2Z, n_raw, ri, nc, n_batch, &pf)) == MMA_OK &&
        (rc = get_plan(CUFFT_Z2D, n2, nc2, ro, n_batch, &pb)) == MMA_OK) {
        cufftSetStream(pf, st);
        cufftSetStream(pb, st);
        gather_rows_kernel<<<grid_for(ri * n_batch), 256, 0, st>>>(raw, n_raw, n_raw, rin, ri, n_batch);
        if (cufftExecD2Z(pf, (cufftDoubleReal*)rin, (cufftDoubleComplex*)spec) != CUFFT_SUCCESS) rc = MMA_ERR_CUFFT;
        if (rc == MMA_OK) {
            pad_scale_kernel<<<grid_for((long long)nc2 * n_batch), 256, 0, st>>>(spec, nc, pad, nc2, n_batch,
                                                                                  1.0 / n_raw);
            if (cufftExecZ2D(pb, (cufftDoubleComplex*)pad, (cufftDoubleReal*)rout) != CUFFT_SUCCESS)
                rc = MMA_ERR_CUFFT;
        }
        if (rc == MMA_OK)
            gather_rows_kernel<<<grid_for((long long)n2 * n_batch), 256, 0, st>>>(rout, ro, n2, interp, n2, n_batch);
    }
    if (spec) cudaFreeAsync(spec, st);
    if (pad) cudaFreeAsync(pad, st);
    if (rin) cudaFreeAsync(rin, st);
    if (rout) cudaFreeAsync(rout, st);
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
    // cuFFT wants rows aligned to its complex type: gather into an even-strided buffer.
    const long long rs = (n_out + 1) / 2 * 2;
    double2* spec = nullptr;
    double* rows = nullptr;
    if (cudaMallocAsync((void**)&spec, sizeof(double2) * (size_t)nc * n_batch, st) != cudaSuccess) return MMA_ERR_CUDA;
    if (cudaMallocAsync((void**)&rows, sizeof(double) * (size_t)rs * n_batch, st) != cudaSuccess) {
        cudaFreeAsync(spec, st);
        return MMA_ERR_CUDA;
    }
    gather_rows_kernel<<<grid_for(rs * n_batch), 256, 0, st>>>(series, series_stride, n_out, rows, rs, n_batch);
    cufftHandle pf;
    int rc = get_plan(CUFFT_D2Z, n_out, rs, nc, n_batch, &pf);
    if (rc == MMA_OK) {
        cufftSetStream(pf, st);
        if (cufftExecD2Z(pf, (cufftDoubleReal*)rows, (cufftDoubleComplex*)spec) != CUFFT_SUCCESS) rc = MMA_ERR_CUFFT;
    }
    if (rc == MMA_OK) {
        const double two_pi = 6.283185307179586476925286766559;
        spectrum_kernel<<<grid_for((long long)nc * n_batch), 256, 0, st>>>(
            spec, nc, n_batch, dt / sqrt(two_pi), dt * dt / two_pi, two_pi / tmax, fsig, fsig_stride, fm2,
            fm2_stride, omega);
    }
    cudaFreeAsync(spec, st);
    cudaFreeAsync(rows, st);
    if (rc == MMA_OK && cudaGetLastError() != cudaSuccess) rc = MMA_ERR_CUDA;
    return rc;
}
