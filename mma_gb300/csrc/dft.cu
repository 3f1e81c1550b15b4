// dft.cu -- batched real DFTs in FP64 for the TDSE's Fourier interpolation and spectra and the
// Gabor transforms (the roles FFTW plays in the reference's tools_fftw3.c:24-68, 84-143, 158-213).
//
// Algorithm (conventions in dft.cuh):
//   * even n: the row is packed as L = n/2 complex values z_j = x_2j + i x_2j+1; with Z = DFT_L(z),
//     X_k = (Z_k + conj Z_{L-k})/2 - i e^{-2 pi i k/n} (Z_k - conj Z_{L-k})/2, k = 0 .. L;
//     c2r inverts that packing and takes the inverse DFT_L.  Odd n: a complex row of length n.
//   * DFT_L: Stockham autosort passes with radices 8, 4, 2, 7, 5, 3 when L is 7-smooth.  Pass p
//     (radix R, Ns = the product of the earlier radices): butterfly j < L/R reads a[j + r L/R],
//     multiplies value r by w^{r k} (w = e^{-2 pi i/(Ns R)}, k = j mod Ns), takes the R-point DFT
//     and writes value r to (j / Ns) Ns R + k + r Ns.  Otherwise Bluestein: with the chirp
//     c_j = e^{-i pi j^2/L}, DFT_L(z)_k = c_k (a * b)_k, a_j = z_j c_j, b_m = conj(c_|m|), the
//     cyclic convolution over the smallest 7-smooth M >= 2L - 1, by FFT_M, a product with the
//     precomputed FFT_M(b)/M, and the inverse FFT_M taken as conj(FFT_M(conj(.))).
//   * Tables (twiddles e^{-2 pi i j/M}, chirp, FFT_M(b)/M, packing factors) are computed once per
//     length on the device with sincospi, whose argument is an exact ratio reduced in integers.
//   * Rows whose FFT length M fits a CTA's shared memory (M <= 7168: two buffers of M values) run
//     one CTA per row with every pass in shared memory, from one buffer to the other; two CTA
//     sizes exist (256 and 512 threads), and the plan keeps the faster one for its length, timed
//     on a probe batch when the plan is made.  Longer rows run one launch per pass through global
//     memory.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "../../include/mma_tdse.h"
#include "dft.cuh"

namespace mma {
namespace dft {

constexpr int kMaxPasses = 32;
// Largest FFT length of the shared-memory kernels: two buffers of 16-byte values within a CTA's
// 227 KB of shared memory.
constexpr int kMaxSmemM = 7168;

struct Plan {
    int n, L, M, bluestein, nr, threads;  // threads: 256 or 512 (shared-memory path), 0 (global path)
    int rad[kMaxPasses];
    double2 *tw, *chirp, *bker, *wpost;
    float tuned_ms[2];  // probe-batch time of the 256- and 512-thread kernels (0: not a candidate)
};

// ------------------------------------------------------------------------------ arithmetic
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conjg(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 mul_mi(double2 a) { return make_double2(a.y, -a.x); }  // -i a

// R-point DFTs y_q = sum_r v_r e^{-2 pi i r q / R}, in place; w[m] = e^{-2 pi i m / R} (table
// values) for the m the radix uses: 1 and 3 for radix 8, 1 .. (R-1)/2 for odd R.
template <int R>
struct Bfly;
template <>
struct Bfly<2> {
    __device__ __forceinline__ static void run(double2* v, const double2*)
    {
        const double2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};
template <>
struct Bfly<4> {
    __device__ __forceinline__ static void run(double2* v, const double2*)
    {
        const double2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]), a3 = mul_mi(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        v[1] = cadd(a1, a3);
        v[3] = csub(a1, a3);
    }
};
template <>
struct Bfly<8> {
    __device__ __forceinline__ static void run(double2* v, const double2* w)
    {
        double2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        Bfly<4>::run(e, nullptr);
        Bfly<4>::run(o, nullptr);
        o[1] = cmul(o[1], w[1]);  // e^{-i pi/4}
        o[2] = mul_mi(o[2]);      // e^{-i pi/2}
        o[3] = cmul(o[3], w[3]);  // e^{-3 i pi/4}
#pragma unroll
        for (int q = 0; q < 4; q++) {
            v[q] = cadd(e[q], o[q]);
            v[q + 4] = csub(e[q], o[q]);
        }
    }
};
// odd R: pairs r, R - r: y_q = v_0 + sum_r [cos(2 pi r q/R) (v_r + v_{R-r}) - i sin(2 pi r q/R) (v_r - v_{R-r})]
template <int R>
struct Bfly {
    static_assert(R % 2 == 1, "odd radix");
    __device__ __forceinline__ static void run(double2* v, const double2* w)
    {
        constexpr int H = (R - 1) / 2;
        double2 s[H + 1], d[H + 1];
        double2 y0 = v[0];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            s[r] = cadd(v[r], v[R - r]);
            d[r] = csub(v[r], v[R - r]);
            y0 = cadd(y0, s[r]);
        }
#pragma unroll
        for (int q = 1; q <= H; q++) {
            double2 a = v[0], b = make_double2(0.0, 0.0);
#pragma unroll
            for (int r = 1; r <= H; r++) {
                // (cos, -sin) of 2 pi m / R, m = r q mod R; for m > H from w[R - m] by symmetry
                const int m = (r * q) % R;
                const double c = m <= H ? w[m].x : w[R - m].x, ms = m <= H ? w[m].y : -w[R - m].y;
                a.x += c * s[r].x;
                a.y += c * s[r].y;
                b.x += ms * d[r].x;  // -sin * d
                b.y += ms * d[r].y;
            }
            // -i sin d = i (-sin d): y_q = a + i b', y_{R-q} = a - i b' with b' = -sin d
            v[q] = make_double2(a.x - b.y, a.y + b.x);
            v[R - q] = make_double2(a.x + b.y, a.y - b.x);
        }
        v[0] = y0;
    }
};

template <int R>
__device__ __forceinline__ void load_roots(double2* w, const double2* __restrict__ tw, int M)
{
    if (R == 8) {
        w[1] = __ldg(tw + M / 8);
        w[3] = __ldg(tw + 3 * (M / 8));
    } else if (R % 2 == 1) {
#pragma unroll
        for (int m = 1; m <= (R - 1) / 2; m++) w[m] = __ldg(tw + m * (M / R));
    }
}

// ------------------------------------------------------------------------------ shared-memory FFT
// One Stockham pass from buffer a to buffer b (both in shared memory), one butterfly per thread at a
// time; a barrier ends the pass.
template <int R>
__device__ __forceinline__ void pass_pp(const double2* __restrict__ a, double2* __restrict__ b, int M, int Ns,
                                        const double2* __restrict__ tw)
{
    const int MR = M / R, step = M / (Ns * R);
    double2 w[R];
    load_roots<R>(w, tw, M);
    for (int j = threadIdx.x; j < MR; j += blockDim.x) {
        const int k = j % Ns;
        double2 v[R];
        v[0] = a[j];
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul(a[j + r * MR], __ldg(tw + r * k * step));
        Bfly<R>::run(v, w);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) b[base + r * Ns] = v[r];
    }
    __syncthreads();
}

// FFT_M of buf[0] into buf[0] or buf[1]; returns the buffer holding the result
__device__ __forceinline__ double2* fft_smem(double2* x, double2* y, const Plan& P)
{
    int Ns = 1;
    for (int p = 0; p < P.nr; p++) {
        const int R = P.rad[p];
        switch (R) {
        case 8: pass_pp<8>(x, y, P.M, Ns, P.tw); break;
        case 4: pass_pp<4>(x, y, P.M, Ns, P.tw); break;
        case 2: pass_pp<2>(x, y, P.M, Ns, P.tw); break;
        case 7: pass_pp<7>(x, y, P.M, Ns, P.tw); break;
        case 5: pass_pp<5>(x, y, P.M, Ns, P.tw); break;
        default: pass_pp<3>(x, y, P.M, Ns, P.tw); break;
        }
        Ns *= R;
        double2* t = x;
        x = y;
        y = t;
    }
    return x;
}

// DFT_L of x[0 .. L) (for Bluestein x holds z_j c_j on [0, L) and zeros on [L, M)); returns the
// buffer (x or y) whose [0 .. L) holds the result.
__device__ __noinline__ double2* dft_core(double2* x, double2* y, const Plan& P)
{
    double2* r = fft_smem(x, y, P);
    if (P.bluestein) {
        for (int j = threadIdx.x; j < P.M; j += blockDim.x) r[j] = conjg(cmul(r[j], __ldg(P.bker + j)));
        __syncthreads();
        r = fft_smem(r, r == x ? y : x, P);
        for (int j = threadIdx.x; j < P.L; j += blockDim.x) r[j] = cmul(conjg(r[j]), __ldg(P.chirp + j));
        __syncthreads();
    }
    return r;
}

// input value j of the complex DFT for r2c (the packed row, times the chirp for Bluestein)
__device__ __forceinline__ double2 r2c_in(const Plan& P, const double* xr, int j)
{
    if (j >= P.L) return make_double2(0.0, 0.0);
    double2 z = (P.n % 2 == 0) ? make_double2(xr[2 * j], xr[2 * j + 1]) : make_double2(xr[j], 0.0);
    return P.bluestein ? cmul(z, __ldg(P.chirp + j)) : z;
}

// bin k of the r2c output from Z = DFT_L (zk = Z_{k mod L}, zc = conj Z_{(L-k) mod L})
__device__ __forceinline__ double2 r2c_out(const Plan& P, double2 zk, double2 zc, int k)
{
    const double2 s = cadd(zk, zc), wd = cmul(__ldg(P.wpost + k), csub(zk, zc));
    return make_double2(0.5 * (s.x + wd.y), 0.5 * (s.y - wd.x));  // s/2 - i w d/2
}

// input value k of the complex DFT for c2r: conj of the packed spectrum (inverse by conjugation),
// times the chirp for Bluestein
__device__ __forceinline__ double2 c2r_in(const Plan& P, const double2* Xr, int nb, int k)
{
    if (k >= P.L) return make_double2(0.0, 0.0);
    double2 Z;
    if (P.n % 2 == 0) {
        double2 Xk = k < nb ? Xr[k] : make_double2(0.0, 0.0);
        double2 Xn;
        if (k == 0) {
            Xk.y = 0.0;
            Xn = P.L < nb ? make_double2(Xr[P.L].x, 0.0) : make_double2(0.0, 0.0);
        } else {
            Xn = P.L - k < nb ? conjg(Xr[P.L - k]) : make_double2(0.0, 0.0);
        }
        const double2 s = cadd(Xk, Xn), wd = cmul(conjg(__ldg(P.wpost + k)), csub(Xk, Xn));
        Z = make_double2(s.x - wd.y, s.y + wd.x);  // s + i w d
    } else {
        const int h = P.n / 2;
        if (k <= h) {
            Z = k < nb ? Xr[k] : make_double2(0.0, 0.0);
            if (k == 0) Z.y = 0.0;
        } else {
            Z = P.n - k < nb ? conjg(Xr[P.n - k]) : make_double2(0.0, 0.0);
        }
    }
    Z = conjg(Z);
    return P.bluestein ? cmul(Z, __ldg(P.chirp + k)) : Z;
}

template <int T>
__global__ void __launch_bounds__(T) r2c_smem(Plan P, const double* __restrict__ x, int64_t xs, double2* X,
                                              int64_t Xs, int n_batch)
{
    extern __shared__ double2 sbuf[];  // two buffers of M values
    double2 *b0 = sbuf, *b1 = sbuf + P.M;
    const int t = threadIdx.x, nc = P.n / 2 + 1;
    for (int64_t row = blockIdx.x; row < n_batch; row += gridDim.x) {
        const double* xr = x + row * xs;
        for (int j = t; j < P.M; j += T) b0[j] = r2c_in(P, xr, j);
        __syncthreads();
        const double2* Z = dft_core(b0, b1, P);
        double2* Xr = X + row * Xs;
        if (P.n % 2 == 0) {
            for (int k = t; k < nc; k += T)
                Xr[k] = r2c_out(P, Z[k == P.L ? 0 : k], conjg(Z[k == 0 ? 0 : P.L - k]), k);
        } else {
            for (int k = t; k < nc; k += T) Xr[k] = Z[k];
        }
        __syncthreads();
    }
}

template <int T>
__global__ void __launch_bounds__(T) c2r_smem(Plan P, const double2* __restrict__ X, int64_t Xs, int nb, double* x,
                                              int64_t xs, int n_batch, double scale)
{
    extern __shared__ double2 sbuf[];
    double2 *b0 = sbuf, *b1 = sbuf + P.M;
    const int t = threadIdx.x;
    for (int64_t row = blockIdx.x; row < n_batch; row += gridDim.x) {
        const double2* Xr = X + row * Xs;
        for (int k = t; k < P.M; k += T) b0[k] = c2r_in(P, Xr, nb, k);
        __syncthreads();
        const double2* Z = dft_core(b0, b1, P);
        double* xr = x + row * xs;
        if (P.n % 2 == 0) {
            for (int j = t; j < P.L; j += T) {
                const double2 z = Z[j];  // conj of the inverse DFT value
                xr[2 * j] = scale * z.x;
                xr[2 * j + 1] = -scale * z.y;
            }
        } else {
            for (int j = t; j < P.L; j += T) xr[j] = scale * Z[j].x;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------ global-memory path
template <int R>
__global__ void g_pass(const double2* __restrict__ in, double2* __restrict__ out, int M, int Ns,
                       const double2* __restrict__ tw, int64_t n_batch)
{
    const int MR = M / R, step = M / (Ns * R);
    double2 w[R];
    load_roots<R>(w, tw, M);
    const int64_t total = n_batch * MR;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = e / MR;
        const int j = (int)(e % MR), k = j % Ns;
        const double2* a = in + row * M;
        double2* b = out + row * M;
        double2 v[R];
        v[0] = a[j];
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul(a[j + r * MR], __ldg(tw + r * k * step));
        Bfly<R>::run(v, w);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) b[base + r * Ns] = v[r];
    }
}

__global__ void g_load_r2c(Plan P, const double* __restrict__ x, int64_t xs, double2* buf, int64_t n_batch)
{
    const int64_t total = n_batch * P.M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        buf[e] = r2c_in(P, x + (e / P.M) * xs, (int)(e % P.M));
}

__global__ void g_load_c2r(Plan P, const double2* __restrict__ X, int64_t Xs, int nb, double2* buf, int64_t n_batch)
{
    const int64_t total = n_batch * P.M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        buf[e] = c2r_in(P, X + (e / P.M) * Xs, nb, (int)(e % P.M));
}

__global__ void g_bluestein_mid(Plan P, double2* buf, int64_t n_batch)
{
    const int64_t total = n_batch * P.M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        buf[e] = conjg(cmul(buf[e], __ldg(P.bker + e % P.M)));
}

// Z_j of the DFT_L from the global buffer: direct, or conj(conv_j) c_j after Bluestein
__device__ __forceinline__ double2 g_Z(const Plan& P, const double2* row, int j)
{
    return P.bluestein ? cmul(conjg(row[j]), __ldg(P.chirp + j)) : row[j];
}

__global__ void g_store_r2c(Plan P, const double2* buf, double2* X, int64_t Xs, int64_t n_batch)
{
    const int nc = P.n / 2 + 1;
    const int64_t total = n_batch * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = e / nc;
        const int k = (int)(e % nc);
        const double2* br = buf + row * P.M;
        double2 v;
        if (P.n % 2 == 0)
            v = r2c_out(P, g_Z(P, br, k == P.L ? 0 : k), conjg(g_Z(P, br, k == 0 ? 0 : P.L - k)), k);
        else
            v = g_Z(P, br, k);
        X[row * Xs + k] = v;
    }
}

__global__ void g_store_c2r(Plan P, const double2* buf, double* x, int64_t xs, int64_t n_batch, double scale)
{
    const int64_t total = n_batch * P.L;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = e / P.L;
        const int j = (int)(e % P.L);
        const double2 z = g_Z(P, buf + row * P.M, j);  // conj of the inverse DFT value
        if (P.n % 2 == 0) {
            x[row * xs + 2 * j] = scale * z.x;
            x[row * xs + 2 * j + 1] = -scale * z.y;
        } else {
            x[row * xs + j] = scale * z.x;
        }
    }
}

// ------------------------------------------------------------------------------ tables
__global__ void init_tables(int M, int L, int n, double2* tw, double2* chirp, double2* wpost)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += stride) {
        double s, c;
        sincospi(-2.0 * (double)j / (double)M, &s, &c);
        tw[j] = make_double2(c, s);
    }
    if (chirp)
        for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < L; j += stride) {
            const int64_t q = (j * j) % (2 * (int64_t)L);  // e^{-i pi j^2 / L}, exponent reduced mod 2L
            double s, c;
            sincospi(-(double)q / (double)L, &s, &c);
            chirp[j] = make_double2(c, s);
        }
    if (wpost)
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= L; k += stride) {
            double s, c;
            sincospi(-2.0 * (double)k / (double)n, &s, &c);
            wpost[k] = make_double2(c, s);
        }
}

__global__ void bluestein_b(int M, int L, const double2* chirp, double2* b)
{
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        if (m < L) v = conjg(chirp[m]);
        else if (m > M - L) v = conjg(chirp[M - m]);
        b[m] = v;
    }
}

__global__ void scale_kernel(double2* v, int M, double s)
{
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x)
        v[m] = make_double2(v[m].x * s, v[m].y * s);
}

// ------------------------------------------------------------------------------ host side
bool smooth(int v)
{
    for (int p : {2, 3, 5, 7})
        while (v % p == 0) v /= p;
    return v == 1;
}

int grid_for(int64_t total)
{
    const int64_t b = (total + 255) / 256;
    return (int)(b < 8192 ? (b > 0 ? b : 1) : 8192);
}

// Global passes over n_batch rows of length M: a -> b -> a ...; returns the buffer holding the result.
double2* run_passes(const Plan& P, double2* a, double2* b, int64_t n_batch, cudaStream_t st)
{
    int Ns = 1;
    for (int p = 0; p < P.nr; p++) {
        const int R = P.rad[p];
        const int g = grid_for(n_batch * (P.M / R));
        switch (R) {
        case 8: g_pass<8><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        case 4: g_pass<4><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        case 2: g_pass<2><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        case 7: g_pass<7><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        case 5: g_pass<5><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        default: g_pass<3><<<g, 256, 0, st>>>(a, b, P.M, Ns, P.tw, n_batch); break;
        }
        Ns *= R;
        double2* tmp = a;
        a = b;
        b = tmp;
    }
    return a;
}

int set_smem_attrs()
{
    static int done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MMA_ERR_NO_DEVICE;
    if (dev >= 0 && dev < 64 && done[dev]) return MMA_OK;
    constexpr int bytes = 2 * kMaxSmemM * 16;
    if (cudaFuncSetAttribute(r2c_smem<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
        cudaFuncSetAttribute(c2r_smem<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
        cudaFuncSetAttribute(r2c_smem<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
        cudaFuncSetAttribute(c2r_smem<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
        return MMA_ERR_CUDA;
    if (dev >= 0 && dev < 64) done[dev] = 1;
    return MMA_OK;
}

int launch_r2c_smem(const Plan& P, int threads, const double* x, int64_t xs, double2* X, int64_t Xs, int n_batch,
                    cudaStream_t st)
{
    const int g = n_batch < (1 << 20) ? n_batch : (1 << 20);
    const size_t smem = 2 * (size_t)P.M * sizeof(double2);
    if (threads == 256)
        r2c_smem<256><<<g, 256, smem, st>>>(P, x, xs, X, Xs, n_batch);
    else
        r2c_smem<512><<<g, 512, smem, st>>>(P, x, xs, X, Xs, n_batch);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

std::mutex g_mu;
std::map<std::pair<int, int>, Plan*> g_plans;

void free_plan(Plan* P)
{
    cudaFree(P->tw);
    cudaFree(P->chirp);
    cudaFree(P->bker);
    cudaFree(P->wpost);
    delete P;
}

// Tables on the device, then the CTA size: each valid shared-memory kernel timed on a probe batch
// (32 rows, best of three after a warm-up launch), the faster one kept.
int make_plan(int n, Plan** out)
{
    Plan* P = new Plan();
    P->n = n;
    P->L = (n % 2 == 0) ? n / 2 : n;
    P->bluestein = !smooth(P->L);
    int M = P->L;
    if (P->bluestein) {
        M = 2 * P->L - 1;
        while (!smooth(M)) M++;
    }
    P->M = M;
    int m = M, nr = 0;
    while (m % 8 == 0) { P->rad[nr++] = 8; m /= 8; }
    if (m % 4 == 0) { P->rad[nr++] = 4; m /= 4; }
    if (m % 2 == 0) { P->rad[nr++] = 2; m /= 2; }
    for (int p : {7, 5, 3})
        while (m % p == 0) { P->rad[nr++] = p; m /= p; }
    P->nr = nr;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        delete P;
        return MMA_ERR_CUDA;
    }
    int rc = MMA_OK;
    double2* ta = nullptr;
    double* probe_x = nullptr;
    double2* probe_X = nullptr;
    if (cudaMalloc(&P->tw, sizeof(double2) * M) != cudaSuccess ||
        (P->bluestein && (cudaMalloc(&P->chirp, sizeof(double2) * P->L) != cudaSuccess ||
                          cudaMalloc(&P->bker, sizeof(double2) * M) != cudaSuccess)) ||
        (n % 2 == 0 && cudaMalloc(&P->wpost, sizeof(double2) * (P->L + 1)) != cudaSuccess))
        rc = MMA_ERR_DFT;
    if (rc == MMA_OK) {
        init_tables<<<grid_for(M), 256, 0, st>>>(M, P->L, n, P->tw, P->chirp, P->wpost);
        if (P->bluestein) {
            if (cudaMalloc(&ta, sizeof(double2) * M) != cudaSuccess) {
                rc = MMA_ERR_DFT;
            } else {
                bluestein_b<<<grid_for(M), 256, 0, st>>>(M, P->L, P->chirp, ta);
                double2* r = run_passes(*P, ta, P->bker, 1, st);
                if (r != P->bker) cudaMemcpyAsync(P->bker, r, sizeof(double2) * M, cudaMemcpyDeviceToDevice, st);
                scale_kernel<<<grid_for(M), 256, 0, st>>>(P->bker, M, 1.0 / M);
            }
        }
        if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = MMA_ERR_CUDA;
    }
    P->threads = 0;
    if (rc == MMA_OK && M <= kMaxSmemM && (rc = set_smem_attrs()) == MMA_OK) {
        const int rows = 32;
        const int cand[2] = {256, 512};
        float best = 1e30f;
        if (cudaMalloc(&probe_x, sizeof(double) * (size_t)rows * n) != cudaSuccess ||
            cudaMalloc(&probe_X, sizeof(double2) * (size_t)rows * (n / 2 + 1)) != cudaSuccess ||
            cudaMemsetAsync(probe_x, 0, sizeof(double) * (size_t)rows * n, st) != cudaSuccess)
            rc = MMA_ERR_DFT;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int c = 0; rc == MMA_OK && c < 2; c++) {
            P->tuned_ms[c] = 0.f;
            float t_best = 1e30f;
            for (int rep = 0; rep < 4 && rc == MMA_OK; rep++) {
                cudaEventRecord(e0, st);
                rc = launch_r2c_smem(*P, cand[c], probe_x, n, probe_X, n / 2 + 1, rows, st);
                cudaEventRecord(e1, st);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = MMA_ERR_CUDA;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0 && ms < t_best) t_best = ms;  // the first launch is a warm-up
            }
            P->tuned_ms[c] = t_best;
            if (t_best < best) {
                best = t_best;
                P->threads = cand[c];
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    cudaFree(ta);
    cudaFree(probe_x);
    cudaFree(probe_X);
    cudaStreamDestroy(st);
    if (rc != MMA_OK) {
        free_plan(P);
        return rc;
    }
    *out = P;
    return MMA_OK;
}

int get_plan(int n, cudaStream_t st, const Plan** out)
{
    if (n < 2) return MMA_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MMA_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_pair(dev, n);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        *out = it->second;
        return MMA_OK;
    }
        // a plan allocates and synchronises: refuse while the caller's stream is being captured
    // (the first call for each length must come before any capture)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return MMA_ERR_DFT;
    Plan* P = nullptr;
    const int rc = make_plan(n, &P);
    if (rc != MMA_OK) return rc;
    g_plans[key] = P;
    *out = P;
    return MMA_OK;
}

int r2c(const Plan* p, const double* x, int64_t xs, double2* X, int64_t Xs, int n_batch, cudaStream_t st)
{
    if (!p || !x || !X || n_batch < 1 || xs < p->n || Xs < p->n / 2 + 1) return MMA_ERR_ARG;
    const Plan& P = *p;
    if (P.threads) return launch_r2c_smem(P, P.threads, x, xs, X, Xs, n_batch, st);
    double2 *a = nullptr, *b = nullptr;
    const size_t bytes = sizeof(double2) * (size_t)P.M * n_batch;
    if (cudaMallocAsync((void**)&a, bytes, st) != cudaSuccess) return MMA_ERR_CUDA;
    if (cudaMallocAsync((void**)&b, bytes, st) != cudaSuccess) {
        cudaFreeAsync(a, st);
        return MMA_ERR_CUDA;
    }
    const int64_t nbt = n_batch;
    g_load_r2c<<<grid_for(nbt * P.M), 256, 0, st>>>(P, x, xs, a, nbt);
    double2* r = run_passes(P, a, b, nbt, st);
    if (P.bluestein) {
        g_bluestein_mid<<<grid_for(nbt * P.M), 256, 0, st>>>(P, r, nbt);
        r = run_passes(P, r, r == a ? b : a, nbt, st);
    }
    g_store_r2c<<<grid_for(nbt * (P.n / 2 + 1)), 256, 0, st>>>(P, r, X, Xs, nbt);
    cudaFreeAsync(a, st);
    cudaFreeAsync(b, st);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

int c2r(const Plan* p, const double2* X, int64_t Xs, int n_bins, double* x, int64_t xs, int n_batch, double scale,
        cudaStream_t st)
{
    if (!p || !x || !X || n_batch < 1 || n_bins < 1 || xs < p->n || Xs < n_bins) return MMA_ERR_ARG;
    const Plan& P = *p;
    if (P.threads) {
        const int g = n_batch < (1 << 20) ? n_batch : (1 << 20);
        const size_t smem = 2 * (size_t)P.M * sizeof(double2);
        if (P.threads == 256)
            c2r_smem<256><<<g, 256, smem, st>>>(P, X, Xs, n_bins, x, xs, n_batch, scale);
        else
            c2r_smem<512><<<g, 512, smem, st>>>(P, X, Xs, n_bins, x, xs, n_batch, scale);
        return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
    }
    double2 *a = nullptr, *b = nullptr;
    const size_t bytes = sizeof(double2) * (size_t)P.M * n_batch;
    if (cudaMallocAsync((void**)&a, bytes, st) != cudaSuccess) return MMA_ERR_CUDA;
    if (cudaMallocAsync((void**)&b, bytes, st) != cudaSuccess) {
        cudaFreeAsync(a, st);
        return MMA_ERR_CUDA;
    }
    const int64_t nbt = n_batch;
    g_load_c2r<<<grid_for(nbt * P.M), 256, 0, st>>>(P, X, Xs, n_bins, a, nbt);
    double2* r = run_passes(P, a, b, nbt, st);
    if (P.bluestein) {
        g_bluestein_mid<<<grid_for(nbt * P.M), 256, 0, st>>>(P, r, nbt);
        r = run_passes(P, r, r == a ? b : a, nbt, st);
    }
    g_store_c2r<<<grid_for(nbt * P.L), 256, 0, st>>>(P, r, x, xs, nbt, scale);
    cudaFreeAsync(a, st);
    cudaFreeAsync(b, st);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

}  // namespace dft
}  // namespace mma

using namespace mma;

// Plan facts for a real DFT of length n (creating the plan): the complex FFT length M, whether
// Bluestein's convolution is used, the CTA size the plan runs (0: the global-memory path) and the
// probe-batch times of the 256- and 512-thread kernels in ms (0 where not a candidate).
extern "C" int mma_dft_plan_info(int n, int* fft_len, int* bluestein, int* cta_threads, float* probe_ms)
{
    const dft::Plan* P = nullptr;
    const int rc = dft::get_plan(n, nullptr, &P);
    if (rc != MMA_OK) return rc;
    if (fft_len) *fft_len = P->M;
    if (bluestein) *bluestein = P->bluestein;
    if (cta_threads) *cta_threads = P->threads;
    if (probe_ms) {
        probe_ms[0] = P->tuned_ms[0];
        probe_ms[1] = P->tuned_ms[1];
    }
    return MMA_OK;
}

extern "C" int mma_dft_r2c(int n, const double* x, int64_t x_stride, double* X, int64_t X_stride, int n_batch,
                           void* stream)
{
    if (n < 2 || !x || !X || n_batch < 1) return MMA_ERR_ARG;
    const dft::Plan* P = nullptr;
    const int rc = dft::get_plan(n, (cudaStream_t)stream, &P);
    if (rc != MMA_OK) return rc;
    return dft::r2c(P, x, x_stride, reinterpret_cast<double2*>(X), X_stride, n_batch, (cudaStream_t)stream);
}

extern "C" int mma_dft_c2r(int n, const double* X, int64_t X_stride, int n_bins, double* x, int64_t x_stride,
                           int n_batch, double scale, void* stream)
{
    if (n < 2 || !x || !X || n_batch < 1) return MMA_ERR_ARG;
    const dft::Plan* P = nullptr;
    const int rc = dft::get_plan(n, (cudaStream_t)stream, &P);
    if (rc != MMA_OK) return rc;
    return dft::c2r(P, reinterpret_cast<const double2*>(X), X_stride, n_bins, x, x_stride, n_batch, scale,
                    (cudaStream_t)stream);
}
