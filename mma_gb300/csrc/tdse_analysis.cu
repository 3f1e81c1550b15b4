// tdse_analysis.cu -- analysis kernels of the TDSE library, batched on the GPU:
//   * the photoelectron spectrum by the resolvent window method (1DTDSE/sources/tools.c:206-316,
//     window_analysis): for every energy E_i two complex Numerov-tridiagonal solves,
//       (M2 (E_i - dE - i dE - V) - K) u1 = M2 psi,   (M2 (E_i + dE + i dE - V) - K) u2 = M2 u1,
//       PES_i = dx dE^4 sum_j |u2_j|^2,
//     one thread per energy, each a serial FP64 Thomas sweep (tridiag.c:26-70, 251-274) with its
//     elimination factors interleaved across energies so that a warp's loads coalesce;
//   * the Gabor transform (tools_fftw3.c:158-213, GaborTransform): for every window centre
//     t_w = t_min + w (t_max - t_min)/N_G the signal times exp(-((t_j - t_w)/a)^2), a real DFT
//     (this library's own, dft.cu, batched over windows and signals) and dt/sqrt(2 pi) |DFT_k| for
//     k < N_freq.
// The arithmetic follows the reference's expressions and their order (FP64).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>

#include "../../include/mma_tdse.h"
#include "common.cuh"
#include "dft.cuh"

namespace mma {
namespace an {

constexpr double kPi = 3.14159265358979323846;

// Energy-independent tables of the photoelectron spectrum: x_k = k dx - xmax with
// xmax = 0.5 num_r dx (tools.c:231, 246), V(x_k) = -1/sqrt(a^2 + x^2) (tools.c:91-95) kept as
// V/12 (n + 1 entries: the reference reads x[num_r + 1] for an unused super-diagonal of the
// last row), and the right-hand side of the first solve, M2 psi = (10 psi_j + psi_{j-1} +
// psi_{j+1})/12 (tridiag.c:261-268), which is the same for every energy.
__global__ void pes_tables(int64_t n, int num_r, double dx, double a, const double* psi, double* V12, cd* rhs0)
{
    const double xmax = __dmul_rn(__dmul_rn(0.5, (double)num_r), dx);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= n; k += (int64_t)gridDim.x * blockDim.x) {
        const double x = __dsub_rn(__dmul_rn((double)k, dx), xmax);
        V12[k] = (-1.0 / sqrt(a * a + x * x)) / 12.;
        if (k < n) {
            const cd pc{psi[2 * k], psi[2 * k + 1]};
            const cd pm = k > 0 ? cd{psi[2 * k - 2], psi[2 * k - 1]} : cd{0.0, 0.0};
            const cd pn = k + 1 < n ? cd{psi[2 * k + 2], psi[2 * k + 3]} : cd{0.0, 0.0};
            rhs0[k] = cd{10 * pc.re / 12. + (pn.re + pm.re) / 12., 10 * pc.im / 12. + (pn.im + pm.im) / 12.};
        }
    }
}

struct PesArgs {
    int64_t n;        // rows = num_r + 1
    double dx, dE, Estep, E_start;
    int num_E, e0, chunk;
    const double* V12;  // [n + 1]  V / 12
    const cd* rhs0;     // [n]      M2 psi
    cd* gam;            // [n][chunk]
    cd* u;              // [n][chunk]
    double* pes;        // [num_E]
};

// One Numerov-tridiagonal solve for the energy of this thread (sg = -1: first window, +1:
// second).  Rows of (M2 (Es -/+ i dE - V) - K): diagonal 10 (Es - V_j)/12 - 1/dx^2 -/+ i 10 dE/12,
// sub-diagonal of row j (Es - V_{j-1})/12 + 0.5/dx^2 -/+ i dE/12, super-diagonal of row j-1
// (Es - V_j)/12 + 0.5/dx^2 -/+ i dE/12 (tools.c:257-275).  The right-hand side is M2 psi (first
// solve) or M2 u1 formed from the first solve's result, which the sweep overwrites row by row
// after reading it.  The Thomas recurrence is that of tridiag.c:26-70 with one reciprocal of
// |beta|^2 per row; Es/12 and V/12 are formed once, so the rows need no divisions.
__device__ __forceinline__ void pes_solve(const PesArgs& A, int e, double E, double sg, bool rhs_from_u,
                                          double* norm_out)
{
    const int64_t n = A.n, C = A.chunk;
    const double Es = E + sg * A.dE;  // E_start + Estep i -/+ dE
    const double e12 = Es / 12., e10 = 10 * Es / 12.;
    const double diag = 1. / (A.dx * A.dx), off = -0.5 / (A.dx * A.dx);
    const double im_d = (sg < 0 ? -1.0 : 1.0) * (10 * A.dE / 12), im_o = (sg < 0 ? -1.0 : 1.0) * (A.dE / 12);
    constexpr double k12 = 1.0 / 12.;
    cd pm{0.0, 0.0}, pc{0.0, 0.0}, pn{0.0, 0.0};
    if (rhs_from_u) {
        pc = A.u[e];
        pn = (n > 1) ? A.u[C + e] : cd{0.0, 0.0};
    }
    auto rhs = [&](int64_t j) -> cd {
        if (!rhs_from_u) return A.rhs0[j];
        return cd{(10 * pc.re + (pn.re + pm.re)) * k12, (10 * pc.im + (pn.im + pm.im)) * k12};
    };
    // row 0
    cd r = rhs(0);
    double v12 = A.V12[0];
    double b_re = (e10 - 10 * v12) - diag, b_im = im_d;
    double bet_re = b_re, bet_im = b_im;
    double inv = 1.0 / (bet_re * bet_re + bet_im * bet_im);
    cd uprev{(r.re * b_re + r.im * b_im) * inv, (r.im * b_re - r.re * b_im) * inv};
    A.u[e] = uprev;
    for (int64_t j = 1; j < n; j++) {
        if (rhs_from_u) {
            pm = pc;
            pc = pn;
            pn = (j + 1 < n) ? A.u[(j + 1) * C + e] : cd{0.0, 0.0};
        }
        r = rhs(j);
        const double v12j = A.V12[j];
        const double a_re = (e12 - v12) - off, a_im = im_o;   // dinf[j-1]
        const double c_re = (e12 - v12j) - off, c_im = im_o;  // dsup[j-1]
        const double g_re = (c_re * bet_re + c_im * bet_im) * inv;
        const double g_im = (c_im * bet_re - c_re * bet_im) * inv;
        A.gam[j * C + e] = cd{g_re, g_im};
        b_re = (e10 - 10 * v12j) - diag;
        bet_re = b_re - (a_re * g_re - a_im * g_im);
        bet_im = b_im - (a_im * g_re + a_re * g_im);
        inv = 1.0 / (bet_re * bet_re + bet_im * bet_im);
        const double t_re = r.re - a_re * uprev.re + a_im * uprev.im;
        const double t_im = r.im - a_re * uprev.im - a_im * uprev.re;
        uprev = cd{(t_re * bet_re + t_im * bet_im) * inv, (-t_re * bet_im + t_im * bet_re) * inv};
        A.u[j * C + e] = uprev;  // the rhs of row j+1 already holds u1_j (pc) and u1_{j+1} (pn)
        v12 = v12j;
    }
    // back substitution (tridiag.c:62-66)
    cd unext = uprev;
    double nrm = unext.re * unext.re + unext.im * unext.im;
    for (int64_t j = n - 2; j >= 0; j--) {
        const cd g = A.gam[(j + 1) * C + e];
        cd uj = A.u[j * C + e];
        uj.re -= g.re * unext.re - g.im * unext.im;
        uj.im -= g.re * unext.im + g.im * unext.re;
        A.u[j * C + e] = uj;
        nrm += uj.re * uj.re + uj.im * uj.im;
        unext = uj;
    }
    *norm_out = nrm;
}

__global__ void __launch_bounds__(64) pes_kernel(PesArgs A)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int ie = A.e0 + e;
    if (e >= A.chunk || ie >= A.num_E) return;
    const double E = A.E_start + A.Estep * ie;
    double nrm;
    pes_solve(A, e, E, -1.0, false, &nrm);
    pes_solve(A, e, E, +1.0, true, &nrm);
    A.pes[ie] = nrm * A.dx * pow(A.dE, 4.);
}

// Gabor windows exp(-(ia (j dt - (t_min + w dt_G)))^2) (tools_fftw3.c:180-196, ia = 1/a), the
// same for every signal: tabulated once per call, [N_G][N]
__global__ void gabor_table(int N, int N_G, double dt, double t_min, double dt_G, double ia, double* win)
{
    const int64_t total = (int64_t)N_G * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q % N, w = q / N;
        const double arg = ia * (((double)j) * dt - (t_min + ((double)w) * dt_G));
        win[q] = exp(-(arg * arg));  // arg * arg: the correctly rounded square, as pow(arg, 2.)
    }
}

// windowed signals in[(s N_G + w) N + j] = win[w][j] signal_s[j]
__global__ void gabor_window(const double* sig, int64_t stride, int n_sig, int N, int N_G, const double* win,
                             double* in)
{
    const int64_t total = (int64_t)n_sig * N_G * N;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q % N, b = q / N, w = b % N_G, s = b / N_G;
        in[q] = win[w * N + j] * sig[s * stride + j];
    }
}

// |DFT| of the first N_freq bins times dt/sqrt(2 pi) (tools_fftw3.c:203-205)
__global__ void gabor_abs(const double2* out, int64_t Nc, int64_t nb, int N_freq, double norm, double* g)
{
    const int64_t total = nb * N_freq;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = q % N_freq, b = q / N_freq;
        const double2 v = out[b * Nc + k];
        g[q] = norm * sqrt((v.x * v.x + v.y * v.y));
    }
}

int grid_for(int64_t total) { return (int)((total + 255) / 256 < 8192 ? (total + 255) / 256 : 8192); }

}  // namespace an
}  // namespace mma

using namespace mma;


namespace {
// scratch: V/12 [n + 1] | M2 psi [n] | gam [n][chunk] | u [n][chunk]
size_t pes_fixed(size_t n) { return (sizeof(double) * (n + 1) + 255) / 256 * 256 + (sizeof(cd) * n + 255) / 256 * 256; }
}  // namespace

extern "C" size_t mma_tdse_pes_scratch_bytes(int num_r, int chunk)
{
    if (num_r < 1 || chunk < 1) return 0;
    const size_t n = (size_t)num_r + 1;
    return pes_fixed(n) + 2 * sizeof(cd) * n * (size_t)chunk;
}

extern "C" int mma_tdse_pes(const double* psi, int num_r, double dx, double trg_a, int num_E, double dE, double Estep,
                            double E_start, double* pes, void* scratch, size_t scratch_bytes, void* stream)
{
    if (!psi || !pes || !scratch || num_r < 1 || num_E < 1 || !(dx > 0.0)) return MMA_ERR_ARG;
    const int64_t n = (int64_t)num_r + 1;
    const size_t fixed = pes_fixed((size_t)n);
    if (scratch_bytes < fixed + 2 * sizeof(cd) * (size_t)n) return MMA_ERR_ARG;
    int64_t chunk = (int64_t)((scratch_bytes - fixed) / (2 * sizeof(cd) * (size_t)n));
    if (chunk > num_E) chunk = num_E;
    cudaStream_t st = (cudaStream_t)stream;
    char* sc = static_cast<char*>(scratch);
    double* V12 = reinterpret_cast<double*>(sc);
    cd* rhs0 = reinterpret_cast<cd*>(sc + (sizeof(double) * (size_t)(n + 1) + 255) / 256 * 256);
    cd* gam = reinterpret_cast<cd*>(sc + fixed);
    cd* u = gam + (size_t)n * chunk;
    an::pes_tables<<<an::grid_for(n + 1), 256, 0, st>>>(n, num_r, dx, trg_a, psi, V12, rhs0);
    for (int e0 = 0; e0 < num_E; e0 += (int)chunk) {
        an::PesArgs A{n, dx, dE, Estep, E_start, num_E, e0, (int)chunk, V12, rhs0, gam, u, pes};
        const int cnt = (int)((num_E - e0 < chunk) ? num_E - e0 : chunk);
        an::pes_kernel<<<(cnt + 63) / 64, 64, 0, st>>>(A);  // small blocks: few energies still reach every SM
    }
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

extern "C" size_t mma_gabor_scratch_bytes(int n_sig, int N, int N_G)
{
    if (n_sig < 1 || N < 2 || N_G < 1) return 0;
    const size_t nb = (size_t)n_sig * N_G, Nc = (size_t)N / 2 + 1;
    return (sizeof(double) * nb * N + 255) / 256 * 256 + sizeof(double2) * nb * Nc;
}

extern "C" int mma_gabor(const double* signals, int64_t stride, int n_sig, double dt, int N, int N_freq, int N_G,
                         double t_min, double t_max, double a, double* gabor, void* scratch, size_t scratch_bytes,
                         void* stream)
{
    if (!signals || !gabor || !scratch || n_sig < 1 || N < 2 || N_G < 1 || N_freq < 1 || stride < N) return MMA_ERR_ARG;
    const int64_t Nc = N / 2 + 1;
    if (N_freq > Nc || !(a != 0.0)) return MMA_ERR_ARG;
    if (scratch_bytes < mma_gabor_scratch_bytes(n_sig, N, N_G)) return MMA_ERR_ARG;
    if ((int64_t)n_sig * N_G > 2147483647LL) return MMA_ERR_TOO_LARGE;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nb = (int64_t)n_sig * N_G;
    double* in = static_cast<double*>(scratch);
    double2* out = reinterpret_cast<double2*>(static_cast<char*>(scratch) + (sizeof(double) * nb * N + 255) / 256 * 256);
    const double ia = 1.0 / a, dt_G = (t_max - t_min) / N_G;
    // the window table sits at the front of the DFT output buffer: it is read before the DFT writes there
    double* win = reinterpret_cast<double*>(out);
    an::gabor_table<<<an::grid_for((int64_t)N_G * N), 256, 0, st>>>(N, N_G, dt, t_min, dt_G, ia, win);
    an::gabor_window<<<an::grid_for(nb * N), 256, 0, st>>>(signals, stride, n_sig, N, N_G, win, in);
    const mma::dft::Plan* p = nullptr;
    int rc = mma::dft::get_plan(N, st, &p);
    if (rc == MMA_OK) rc = mma::dft::r2c(p, in, N, out, Nc, (int)nb, st);
    if (rc != MMA_OK) return rc;
    an::gabor_abs<<<an::grid_for(nb * N_freq), 256, 0, st>>>(out, Nc, nb, N_freq, dt / sqrt(2. * an::kPi), gabor);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
