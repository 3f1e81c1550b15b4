// tdse_adjoint.cu -- gradient of a band-limited harmonic yield with respect to the driving
// field: the adjoint of the FP64 Crank-Nicolson-Numerov propagation (the differentiable form).
//
// Forward model of one instance (tdse_step.cuh; reference 1DTDSE/sources/prop.c:115-347):
//   psi_{k+1} = Phi_k U psi_k,   U = 2 A^{-1} M2 - I,   Phi_k = diag(e^{i F_k dt x_j}),
//   s_{k+1}   = -sum_j |psi_{k+1,j}|^2 gv_j + F_k          (sourceterm, gv = -V')
//   L         = dt^2/(2 pi) sum_{q in Q} |D_q|^2,  D_q = sum_{n<S} s_n e^{-2 pi i q n / S}
// With lambda = dL/dRe psi + i dL/dIm psi and a_n = dL/ds_n:
//   lambda_S = 0 (s_S is not a spectrum sample),
//   dL/dF_k  = a_{k+1} - dt sum_j x_j Im(conj(lambda_{k+1,j}) psi_{k+1,j})
//   lambda_k = U^H Phi_k^H lambda_{k+1} - 2 a_k gv .* psi_k,   U^H mu = 2 M2 (A^H)^{-1} mu - mu,
// A^H solved with its own factorisation (build_grids_kernel, adj_tab) by the same
// partitioned solve.  The forward pass stores psi every K steps (ckpt_*); going backwards,
// each segment is recomputed forwards from its checkpoint into a per-CTA history, then
// swept backwards.  Cost: about three forward passes.
#include <cuda_runtime.h>

#include "../../include/mma_tdse.h"
#include "common.cuh"
#include "tdse_solver.cuh"
#include "tdse_step.cuh"

namespace mma {
namespace adj {

constexpr double kTwoPi = 6.283185307179586476925286766559;

// ---------------------------------------------------------------------------- loss gradient
// One CTA per instance: D_q over the band by direct sums (angle 2 pi (q n mod S)/S, exact
// integer reduction), L, then a_n = 2 c2 Re(sum_q D_q e^{+2 pi i q n / S}).
__global__ void __launch_bounds__(kThreads) loss_grad_kernel(const mma_tdse_instance* insts, const double* outputs,
                                                             const double* tmax, double dt, double w_lo,
                                                             double w_hi, double* loss, double* a,
                                                             const int64_t* a_off)
{
    extern __shared__ double2 Dq[];  // band coefficients
    __shared__ double red[kWarps];
    const mma_tdse_instance I = insts[blockIdx.x];
    const int64_t S = I.n_steps;
    const double* s = outputs + I.out_off + 2 * (S + 1);
    const double tm = tmax[blockIdx.x];
    int64_t q_lo = (int64_t)ceil(w_lo * tm / kTwoPi), q_hi = (int64_t)floor(w_hi * tm / kTwoPi);
    if (q_lo < 1) q_lo = 1;
    if (q_hi > S / 2) q_hi = S / 2;
    const int64_t nq = q_hi >= q_lo ? q_hi - q_lo + 1 : 0;
    const double c2 = dt * dt / kTwoPi;
    double part = 0.0;
    for (int64_t iq = threadIdx.x; iq < nq; iq += blockDim.x) {
        const int64_t q = q_lo + iq;
        double re = 0.0, im = 0.0;
        for (int64_t n = 0; n < S; n++) {
            double sn, cs;
            sincospi(2.0 * (double)((q * n) % S) / (double)S, &sn, &cs);
            re = fma(s[n], cs, re);
            im = fma(-s[n], sn, im);
        }
        Dq[iq] = make_double2(re, im);
        part += c2 * (re * re + im * im);
    }
    double v[1] = {part};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) loss[blockIdx.x] = v[0];
    double* ai = a + a_off[blockIdx.x];
    for (int64_t n = threadIdx.x; n <= S; n += blockDim.x) {
        double acc = 0.0;
        if (n < S)
            for (int64_t iq = 0; iq < nq; iq++) {
                const int64_t q = q_lo + iq;
                double sn, cs;
                sincospi(2.0 * (double)((q * n) % S) / (double)S, &sn, &cs);
                acc = fma(Dq[iq].x, cs, fma(-Dq[iq].y, sn, acc));
            }
        ai[n] = 2.0 * c2 * acc;
    }
}

// ---------------------------------------------------------------------------- adjoint sweep
struct Args {
    const mma_tdse_instance* insts;
    int n_inst;
    const mma_tdse_grid* grids;
    const double* fields;
    const double* ckpts;
    const double* a;
    const int64_t* a_off;
    double* grad;
    const int64_t* grad_off;
    int* counter;
    cd* scratch;  // per CTA: yl [max_L], history [(max_K + 1) max_L]
    int64_t max_L, max_K;
};

__global__ void __launch_bounds__(kThreads, 1) adjoint_fp64_kernel(Args P)
{
    extern __shared__ double2 smem_dyn[];
    cd* lam = reinterpret_cast<cd*>(smem_dyn);  // lambda, chunk-interleaved, [L]
    __shared__ cd sc[2 * kWarps], sb[2 * kWarps];
    __shared__ double red[kWarps];
    __shared__ int64_t s_inst, s_gate;
    const int t = threadIdx.x;
    cd* yl = P.scratch + (int64_t)blockIdx.x * (P.max_K + 2) * P.max_L;
    cd* hist = yl + P.max_L;

    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        const int64_t n = G.n, m = G.m, L = m * kThreads, S = I.n_steps, K = I.ckpt_every;
        const cd* ctab = reinterpret_cast<const cd*>(G.cn_tab);
        const cd* atab = reinterpret_cast<const cd*>(G.adj_tab);
        const cd *GVX = ctab + CN_GVX * L;
        const cd *aib = atab + CN_IB6 * L, *ah = atab + CN_H * L, *aF = atab + CN_F * L, *ag = atab + CN_G * L,
                 *aG = atab + CN_GG * L;
        const double* f = P.fields + I.field_off;
        const double* ai = P.a + P.a_off[inst];
        double* gi = P.grad + P.grad_off[inst];
        const double dt = G.dt, dx = G.dx;
        if (t == 0) s_gate = gate_index(f, I.n_field, S, I.gate_floor);
        for (int64_t i = 0; i < m; i++) lam[i * kThreads + t] = cd{0.0, 0.0};  // lambda_S = 0
        __syncthreads();
        const int64_t gate = s_gate;
        const int64_t s0 = t * m;
        const double xs = (s0 < n) ? GVX[t].im : 0.0;
        auto field = [&](int64_t k) { return (k <= gate || k >= I.n_field) ? 0.0 : f[k]; };
        const int64_t nseg = (S + K - 1) / K;
        for (int64_t c = nseg - 1; c >= 0; c--) {
            const int64_t k0 = c * K, k1 = (k0 + K < S) ? k0 + K : S;
            // ---- recompute states k0 .. k1 into the history (hist[h] = psi_{k0+h})
            const double* cp = P.ckpts + I.ckpt_off + c * 2 * n;
            for (int64_t i = 0; i < m; i++) {
                const int64_t j = s0 + i;
                hist[i * kThreads + t] = (j < n) ? ld2(cp + 2 * j) : cd{0.0, 0.0};
            }
            __syncthreads();
            for (int64_t k = k0; k < k1; k++) {
                cd* cur = hist + (k - k0) * P.max_L;
                cd* nxt = cur + P.max_L;
                for (int64_t i = 0; i < m; i++) nxt[i * kThreads + t] = cur[i * kThreads + t];
                __syncthreads();
                cn_step_fp64(nxt, yl, ctab, m, L, field(k), dt, dx, xs, sc, sb, [](int64_t, int64_t, const cd&) {});
                __syncthreads();
            }
            // ---- adjoint steps k = k1-1 .. k0
            for (int64_t k = k1 - 1; k >= k0; k--) {
                const cd* pnext = hist + (k + 1 - k0) * P.max_L;
                const cd* pcur = hist + (k - k0) * P.max_L;
                const double Fk = field(k);
                double sn, cs;
                sincos(Fk * dt * xs, &sn, &cs);
                cd ph{cs, sn};
                sincos(Fk * dt * dx, &sn, &cs);
                const cd z{cs, sn};
                // pass A: gradient term, mu = conj(Phi) lambda, forward sweep of A^H z = mu
                double gsum = 0.0;
                cd yprev{0.0, 0.0};
                for (int64_t i = 0; i < m; i++) {
                    const int64_t q = i * kThreads + t;
                    const cd l = lam[q], p = pnext[q];
                    gsum = fma(GVX[q].im, l.re * p.im - l.im * p.re, gsum);  // x Im(conj(l) p)
                    const cd mu{fma(ph.re, l.re, ph.im * l.im), fma(ph.re, l.im, -ph.im * l.re)};
                    ph = cmul(ph, z);
                    lam[q] = mu;
                    const cd y = cfms(ah[q], yprev, cmul(aib[q], mu));
                    yl[q] = y;
                    yprev = y;
                }
                const cd yin = scan_forward<cd>(aF[(m - 1) * kThreads + t], yprev, sc, sb);
                cd unext{0.0, 0.0};
                for (int64_t i = m - 1; i >= 0; i--) {
                    const int64_t q = i * kThreads + t;
                    const cd y = cfma(aF[q], yin, yl[q]);
                    const cd u = cfms(ag[q], unext, y);
                    yl[q] = u;
                    unext = u;
                }
                const cd uin = scan_backward<cd>(aG[t], unext, sc + kWarps, sb + kWarps);
                for (int64_t i = 0; i < m; i++) {
                    const int64_t q = i * kThreads + t;
                    yl[q] = cfma(aG[q], uin, yl[q]);  // z = (A^H)^{-1} mu
                }
                double v[1] = {gsum};
                block_sum<1>(v, red);  // also orders the z writes before the neighbour reads
                if (t == 0) gi[k] = ai[k + 1] - dt * v[0];
                // pass D: lambda_k = 2 M2 z - mu - 2 a_k gv psi_k  (2 M2 z = (z_- + 10 z + z_+)/6)
                const double ak = ai[k];
                cd zm = (t == 0) ? cd{0.0, 0.0} : yl[(m - 1) * kThreads + t - 1];
                cd zc = yl[t];
                for (int64_t i = 0; i < m; i++) {
                    const int64_t q = i * kThreads + t;
                    const cd zn = (i + 1 < m) ? yl[q + kThreads] : ((t + 1 < kThreads) ? yl[t + 1] : cd{0.0, 0.0});
                    const cd mu = lam[q], p = pcur[q];
                    const double w = -2.0 * ak * GVX[q].re;
                    cd l{(zm.re + zn.re + 10.0 * zc.re) / 6.0 - mu.re + w * p.re,
                         (zm.im + zn.im + 10.0 * zc.im) / 6.0 - mu.im + w * p.im};
                    if (s0 + i >= n) l = cd{0.0, 0.0};
                    lam[q] = l;
                    zm = zc;
                    zc = zn;
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

}  // namespace adj
}  // namespace mma

using namespace mma;

extern "C" int mma_tdse_loss_grad(const mma_tdse_instance* insts, int n_inst, const double* outputs,
                                  const double* tmax, double dt, double w_lo, double w_hi, double* loss, double* a,
                                  const int64_t* a_off, void* stream)
{
    if (n_inst <= 0) return MMA_OK;
    if (!insts || !outputs || !tmax || !loss || !a || !a_off || !(dt > 0.0) || !(w_hi >= w_lo)) return MMA_ERR_ARG;
    // the band holds at most S/2 bins; 12288 bins of shared memory cover S <= 24576
    const size_t smem = sizeof(double2) * 12288;
    cudaFuncSetAttribute(adj::loss_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    adj::loss_grad_kernel<<<n_inst, kThreads, smem, (cudaStream_t)stream>>>(insts, outputs, tmax, dt, w_lo, w_hi,
                                                                           loss, a, a_off);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

extern "C" size_t mma_tdse_adjoint_scratch_bytes(int max_m, int max_ckpt_every, int grid_ctas)
{
    if (grid_ctas <= 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid_ctas = sms > 0 ? sms : 1;
    }
    const size_t L = (size_t)max_m * kThreads;
    return sizeof(cd) * L * ((size_t)max_ckpt_every + 2) * (size_t)grid_ctas;
}

extern "C" int mma_tdse_adjoint(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                const mma_tdse_buffers* bufs, const double* a, const int64_t* a_off, double* grad,
                                const int64_t* grad_off, int max_m, int max_ckpt_every, int grid_ctas, void* stream)
{
    if (n_inst <= 0) return MMA_OK;
    if (!insts || !grids || !bufs || !bufs->fields || !bufs->snapshots || !bufs->counter || !bufs->scratch || !a ||
        !a_off || !grad || !grad_off || max_m < 1 || max_ckpt_every < 1)
        return MMA_ERR_ARG;
    const size_t smem = (size_t)max_m * kThreads * sizeof(cd);
    if (smem > 220 * 1024) return MMA_ERR_TOO_LARGE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MMA_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (grid_ctas <= 0) grid_ctas = sms;
    if (grid_ctas > n_inst) grid_ctas = n_inst;
    if (bufs->scratch_bytes < mma_tdse_adjoint_scratch_bytes(max_m, max_ckpt_every, grid_ctas)) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(bufs->counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    adj::Args A{insts, n_inst, grids, bufs->fields, bufs->snapshots, a, a_off, grad, grad_off, bufs->counter,
                reinterpret_cast<cd*>(bufs->scratch), (int64_t)max_m * kThreads, (int64_t)max_ckpt_every};
    cudaFuncSetAttribute(adj::adjoint_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    adj::adjoint_fp64_kernel<<<grid_ctas, kThreads, smem, st>>>(A);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
