// tdse_kernels.cu -- GB300 kernels for the 1D-TDSE single-atom response.
//
//   build_grids_kernel     grid, -V', ground state (inverse iteration) and the solve
//                          tables of each grid; one CTA per grid.
//   propagate_fp64_kernel  the Crank-Nicolson-Numerov propagation in FP64, one
//                          persistent CTA per instance pulled from a device work
//                          queue, wavefunction resident in shared memory for the
//                          whole pulse, observables reduced in-kernel every step.
//
// Reference map (1DTDSE/sources):
//   grid                 tools.c:62-79            x_k = k dx - num_r dx/2
//   potential, gradient  tools.c:91-113           V = -(a^2+x^2)^-1/2, -V' = x (a^2+x^2)^-3/2
//   ground state         tridiag.c:86-238,251-274 inverse iteration with (K - Eg M2), M2 psi rhs
//   CN-Numerov step      prop.c:137-205           (M2 + i dt/2 K) psi' = (M2 - i dt/2 K) psi, phase e^{+iE dt x}
//   observables          prop.c:293-347           |<psi0|psi>|^2, window population, <x>, -<V'> + E
//   zero gate, time grid prop.c:118-134,241-242
#include <cuda_runtime.h>

#include "../../include/mma_tdse.h"
#include "common.cuh"
#include "tdse_solver.cuh"
#include "tdse_step.cuh"

namespace mma {

// ------------------------------------------------------------------------------------------
// Sequential factorisation of one tridiagonal matrix (thread 0), results chunk-interleaved.
// Row j: sub a_j (column j-1), diagonal b_j, super c_j (column j+1).
// ------------------------------------------------------------------------------------------
template <typename T, typename RowFn>
__device__ void factorise(int64_t n, int64_t m, T* ib, T* h, T* g, double rhs_scale, RowFn row)
{
    T a, b, c, beta, ibeta;
    row(0, a, b, c);
    beta = b;
    T one;
    if constexpr (sizeof(T) == sizeof(double)) one = 1.0; else one = cd{1.0, 0.0};
    for (int64_t j = 0; j < n; j++) {
        T aj, bj, cj;
        row(j, aj, bj, cj);
        if (j > 0) {
            // gamma_j = c_{j-1}/beta_{j-1} ; beta_j = b_j - a_j gamma_j
            T gam;
            if constexpr (sizeof(T) == sizeof(double)) gam = c / beta; else gam = cdiv(c, beta);
            g[qidx(j - 1, m)] = gam;
            if constexpr (sizeof(T) == sizeof(double)) beta = bj - aj * gam; else beta = bj - cmul(aj, gam);
        }
        if constexpr (sizeof(T) == sizeof(double)) {
            ibeta = 1.0 / beta;
            ib[qidx(j, m)] = ibeta * rhs_scale;
            h[qidx(j, m)] = (j > 0) ? aj * ibeta : 0.0;
        } else {
            ibeta = cdiv(one, beta);
            ib[qidx(j, m)] = cd{ibeta.re * rhs_scale, ibeta.im * rhs_scale};
            h[qidx(j, m)] = (j > 0) ? cmul(aj, ibeta) : cd{0.0, 0.0};
        }
        c = cj;
        a = aj;
    }
    g[qidx(n - 1, m)] = T{};
}

// Chunk products F (forward from the chunk start) and G (backward from the chunk end).
template <typename T>
__device__ void chunk_products(int64_t m, const T* h, const T* g, T* F, T* G)
{
    const int t = threadIdx.x;
    T p;
    if constexpr (sizeof(T) == sizeof(double)) p = 1.0; else p = cd{1.0, 0.0};
    for (int64_t i = 0; i < m; i++) {
        int64_t q = i * kThreads + t;
        T mh;
        if constexpr (sizeof(T) == sizeof(double)) mh = -h[q]; else mh = cd{-h[q].re, -h[q].im};
        p = mul_(p, mh);
        F[q] = p;
    }
    if constexpr (sizeof(T) == sizeof(double)) p = 1.0; else p = cd{1.0, 0.0};
    for (int64_t i = m - 1; i >= 0; i--) {
        int64_t q = i * kThreads + t;
        T mg;
        if constexpr (sizeof(T) == sizeof(double)) mg = -g[q]; else mg = cd{-g[q].re, -g[q].im};
        p = mul_(p, mg);
        G[q] = p;
    }
}

// ------------------------------------------------------------------------------------------
// Ground state by shifted inverse iteration (tridiag.c:86-159): psi <- (K - Eg M2)^-1 M2 psi,
// normalise, Numerov energy quotient; stop when |E - E_old| <= CV.  Real arithmetic: the
// matrix and the start vector psi = 1 are real, so the reference's imaginary parts stay 0.
// ------------------------------------------------------------------------------------------
__device__ void ground_state(const mma_tdse_grid& G, const double* tab, double* psi, double* yl, double* vq,
                             double* red, double* sc, double* sb, double* out_psi0)
{
    const int t = threadIdx.x;
    const int64_t n = G.n, m = G.m, L = m * kThreads;
    const double* ib12 = tab + GS_IB12 * L;
    const double* hh = tab + GS_H * L;
    const double* FF = tab + GS_F * L;
    const double* gg = tab + GS_G * L;
    const double* GG = tab + GS_GG * L;
    const double inv_dx2 = 1.0 / (G.dx * G.dx);
    for (int64_t i = 0; i < m; i++) {
        int64_t j = t * m + i, q = i * kThreads + t;
        psi[q] = (j < n) ? 1.0 : 0.0;  // tools.c:39-42
        vq[q] = (j < n) ? soft_coulomb(G.x[j], G.trg_a) : 0.0;
    }
    __syncthreads();
    double e_old = G.Eguess, energy = G.Eguess, test = 0.0;
    int64_t it = 0;
    int status = MMA_OK;
    for (;;) {
        // ---- solve (K - Eg M2) res = M2 psi
        double pm = (t == 0) ? 0.0 : psi[(m - 1) * kThreads + t - 1];
        double pc = psi[t];
        double yprev = 0.0;
        for (int64_t i = 0; i < m; i++) {
            int64_t q = i * kThreads + t;
            double pn = (i + 1 < m) ? psi[q + kThreads] : ((t + 1 < kThreads) ? psi[t + 1] : 0.0);
            double r = fma(10.0, pc, pm + pn);
            double y = fma(-hh[q], yprev, ib12[q] * r);
            yl[q] = y;
            yprev = y;
            pm = pc;
            pc = pn;
        }
        double yin = scan_forward<double>(FF[(m - 1) * kThreads + t], yprev, sc, sb);
        double unext = 0.0;
        for (int64_t i = m - 1; i >= 0; i--) {
            int64_t q = i * kThreads + t;
            double y = fma(FF[q], yin, yl[q]);
            double u = fma(-gg[q], unext, y);
            yl[q] = u;
            unext = u;
        }
        double uin = scan_backward<double>(GG[t], unext, sc + kWarps, sb + kWarps);
        double s2[1] = {0.0};
        for (int64_t i = 0; i < m; i++) {
            int64_t q = i * kThreads + t;
            double u = fma(GG[q], uin, yl[q]);
            yl[q] = u;
            s2[0] = fma(u, u, s2[0]);
        }
        block_sum<1>(s2, red);  // normalise (tools.c:137-145)
        const double nrm = sqrt(s2[0]);
        for (int64_t i = 0; i < m; i++) {
            int64_t q = i * kThreads + t;
            psi[q] = yl[q] / nrm;
        }
        __syncthreads();
        // ---- energy quotient (tridiag.c:172-238)
        double acc[2] = {0.0, 0.0};
        pm = (t == 0) ? 0.0 : psi[(m - 1) * kThreads + t - 1];
        double vm = (t == 0) ? 0.0 : vq[(m - 1) * kThreads + t - 1];
        pc = psi[t];
        double vc = vq[t];
        for (int64_t i = 0; i < m; i++) {
            int64_t q = i * kThreads + t;
            double pn = (i + 1 < m) ? psi[q + kThreads] : ((t + 1 < kThreads) ? psi[t + 1] : 0.0);
            double vn = (i + 1 < m) ? vq[q + kThreads] : ((t + 1 < kThreads) ? vq[t + 1] : 0.0);
            double kpsi = inv_dx2 * pc - 0.5 * inv_dx2 * (pm + pn) + (10.0 / 12.0) * pc * vc + (pm * vm + pn * vn) / 12.0;
            double mpsi = 10.0 * pc / 12.0 + (pm + pn) / 12.0;
            acc[0] = fma(kpsi, mpsi, acc[0]);
            acc[1] = fma(mpsi, mpsi, acc[1]);
            pm = pc;
            pc = pn;
            vm = vc;
            vc = vn;
        }
        block_sum<2>(acc, red);
        energy = acc[0] / acc[1];
        test = fabs(energy - e_old);
        e_old = energy;
        ++it;
        if (it >= G.max_iter) {
            status = MMA_ERR_GS_NOCONV;
            break;
        }
        if (!(test > G.CV)) break;
    }
    // final normalisation (tridiag.c:150)
    double s2[1] = {0.0};
    for (int64_t i = 0; i < m; i++) {
        int64_t q = i * kThreads + t;
        s2[0] = fma(psi[q], psi[q], s2[0]);
    }
    block_sum<1>(s2, red);
    const double nrm = sqrt(s2[0]);
    for (int64_t i = 0; i < m; i++) {
        int64_t j = t * m + i, q = i * kThreads + t;
        if (j < n) {
            out_psi0[2 * j] = psi[q] / nrm;
            out_psi0[2 * j + 1] = 0.0;
        }
    }
    if (t == 0) {
        G.result[0] = energy;
        G.result[1] = (double)it;
        G.result[2] = (double)status;
        G.result[3] = test;
    }
}

// ------------------------------------------------------------------------------------------
// Grid builder.  mode 0: x, ground state, CN tables.  mode 1: CN tables from the grid's
// existing x and psi0 (a caller-supplied ground state, as the legacy call1DTDSE allows).
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) build_grids_kernel(const mma_tdse_grid* grids, int mode)
{
    __shared__ double red[kWarps * 4];
    __shared__ double sc[2 * kWarps], sb[2 * kWarps];
    const mma_tdse_grid G = grids[blockIdx.x];
    const int t = threadIdx.x;
    const int64_t n = G.n, m = G.m, L = m * kThreads, num_r = n - 1;
    const double dx = G.dx, a = G.trg_a, dt = G.dt;

    if (mode == 0) {
        // separately rounded multiply and subtract, as the reference's x86 build evaluates
        // (double)k dx - xmax (no fused multiply-add)
        const double xmax = __dmul_rn(__dmul_rn(0.5, (double)num_r), dx);
        for (int64_t j = t; j < n; j += kThreads) G.x[j] = __dsub_rn(__dmul_rn((double)j, dx), xmax);
        __syncthreads();
    }
    // V_j into gv[] for the factorisations (gv receives -V' at the end)
    for (int64_t j = t; j < n; j += kThreads) G.gv[j] = soft_coulomb(G.x[j], a);
    __syncthreads();
    const double* V = G.gv;
    if (mode == 0) {
        // ground-state tables (tridiag.c:101-115)
        double* gtab = G.gs_tab;
        for (int64_t q = t; q < GS_SLOTS * L; q += kThreads) gtab[q] = 0.0;
        __syncthreads();
        if (t == 0) {
            const double E = G.Eguess, k0 = -0.5 / (dx * dx), d0 = 1.0 / (dx * dx);
            auto row = [&](int64_t j, double& aj, double& bj, double& cj) {
                const double vj = V[j];
                aj = (j > 0) ? k0 - E / 12.0 + V[j - 1] / 12.0 : 0.0;
                bj = 10.0 * vj / 12.0 + d0 - 10.0 * E / 12.0;
                cj = (j + 1 < n) ? k0 - E / 12.0 + V[j + 1] / 12.0 : 0.0;
            };
            factorise<double>(n, m, gtab + GS_IB12 * L, gtab + GS_H * L, gtab + GS_G * L, 1.0 / 12.0, row);
        }
        __syncthreads();
        chunk_products<double>(m, gtab + GS_H * L, gtab + GS_G * L, gtab + GS_F * L, gtab + GS_GG * L);
        __syncthreads();
        // the CN table area doubles as the ground-state work space (3 L of 2*CN_SLOTS*L)
        double* work = G.cn_tab;
        ground_state(G, gtab, work, work + L, work + 2 * L, red, sc, sb, G.psi0);
        __syncthreads();
    }
    // Crank-Nicolson tables (prop.c:138-159): row j sub (1/12, w_{j-1}), diag (10/12, d_j),
    // super (1/12, w_{j+1}); w_q = dt/2 (-1/(2dx^2) + V_q/12), d_q = dt/2 (1/dx^2 + 10 V_q/12).
    // The right-hand side is 2 M2 psi = (psi_{j-1} + 10 psi_j + psi_{j+1})/6 and the new state
    // is A^{-1}(2 M2 psi) - psi, which equals A^{-1} conj(A) psi because A + conj(A) = 2 M2.
    cd* ctab = reinterpret_cast<cd*>(G.cn_tab);
    for (int64_t q = t; q < CN_SLOTS * L; q += kThreads) ctab[q] = cd{0.0, 0.0};
    __syncthreads();
    if (t == 0) {
        const double hdt = 0.5 * dt;
        auto row = [&](int64_t j, cd& aj, cd& bj, cd& cj) {
            const double vj = V[j];
            aj = (j > 0) ? cd{1.0 / 12.0, hdt * (-0.5 / (dx * dx)) + hdt * 1 / 12. * V[j - 1]} : cd{0.0, 0.0};
            bj = cd{10.0 / 12.0, hdt * (1.0 / (dx * dx)) + hdt * 10 / 12. * vj};
            cj = (j + 1 < n) ? cd{1.0 / 12.0, hdt * (-0.5 / (dx * dx)) + hdt * 1 / 12. * V[j + 1]} : cd{0.0, 0.0};
        };
        factorise<cd>(n, m, ctab + CN_IB6 * L, ctab + CN_H * L, ctab + CN_G * L, 1.0 / 6.0, row);
    }
    __syncthreads();
    chunk_products<cd>(m, ctab + CN_H * L, ctab + CN_G * L, ctab + CN_F * L, ctab + CN_GG * L);
    __syncthreads();
    if (G.adj_tab) {
        // A^H for the adjoint: row j has sub = super = 1/12 - i w_j and diagonal 10/12 - i d_j
        // (the conjugate transpose of A's rows j-1, j, j+1); right-hand side used as is.
        cd* atab = reinterpret_cast<cd*>(G.adj_tab);
        for (int64_t q = t; q < ADJ_SLOTS * L; q += kThreads) atab[q] = cd{0.0, 0.0};
        __syncthreads();
        if (t == 0) {
            const double hdt = 0.5 * dt;
            auto row = [&](int64_t j, cd& aj, cd& bj, cd& cj) {
                const double wj = hdt * (-0.5 / (dx * dx)) + hdt * 1 / 12. * V[j];
                aj = (j > 0) ? cd{1.0 / 12.0, -wj} : cd{0.0, 0.0};
                bj = cd{10.0 / 12.0, -(hdt * (1.0 / (dx * dx)) + hdt * 10 / 12. * V[j])};
                cj = (j + 1 < n) ? cd{1.0 / 12.0, -wj} : cd{0.0, 0.0};
            };
            factorise<cd>(n, m, atab + CN_IB6 * L, atab + CN_H * L, atab + CN_G * L, 1.0, row);
        }
        __syncthreads();
        chunk_products<cd>(m, atab + CN_H * L, atab + CN_G * L, atab + CN_F * L, atab + CN_GG * L);
        __syncthreads();
    }
    for (int64_t j = t; j < n; j += kThreads) G.gv[j] = minus_grad_v(G.x[j], a);
    __syncthreads();
    for (int64_t i = 0; i < m; i++) {
        int64_t j = t * m + i, q = i * kThreads + t;
        if (j < n) {
            ctab[CN_PSI0 * L + q] = cd{G.psi0[2 * j], G.psi0[2 * j + 1]};
            ctab[CN_GVX * L + q] = cd{G.gv[j], G.x[j]};
        }
    }
}

// ------------------------------------------------------------------------------------------
// FP64 propagation.
// ------------------------------------------------------------------------------------------
struct PropArgs {
    const mma_tdse_instance* insts;
    int n_inst;
    const mma_tdse_grid* grids;
    const double* fields;
    double* outputs;
    double* psi_final;
    double* snapshots;
    int* counter;
    double* scratch;  // per CTA: yl [L] complex, then (when psi is not in shared memory) psi [L] complex
    int64_t max_L;
};

template <bool PSI_SMEM>
__global__ void __launch_bounds__(kThreads, 1) propagate_fp64_kernel(PropArgs P)
{
    extern __shared__ double2 smem_dyn[];
    __shared__ cd sc[2 * kWarps], sb[2 * kWarps];
    __shared__ double red[kWarps * 5];
    __shared__ int64_t s_inst, s_gate, s_lo, s_hi;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    cd* yl = reinterpret_cast<cd*>(P.scratch) + blockIdx.x * P.max_L;
    cd* psi = PSI_SMEM ? reinterpret_cast<cd*>(smem_dyn)
                       : reinterpret_cast<cd*>(P.scratch) + (gridDim.x + blockIdx.x) * P.max_L;

    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        const int64_t n = G.n, m = G.m, L = m * kThreads, S = I.n_steps;
        const cd* tab = reinterpret_cast<const cd*>(G.cn_tab);
        const cd *P0 = tab + CN_PSI0 * L, *GVX = tab + CN_GVX * L;
        const double* f = P.fields + I.field_off;
        double* out = P.outputs + I.out_off;
        double *o_t = out, *o_e = out + (S + 1), *o_src = out + 2 * (S + 1), *o_ptot = out + 3 * (S + 1),
               *o_pint = out + 4 * (S + 1), *o_x = out + 5 * (S + 1);
        const double dt = G.dt, dx = G.dx;
        if (L > P.max_L) {
            // A grid with more sites per thread than the launch was sized for (max_m) would
            // overrun this CTA's sweep buffer and its shared memory: the instance is skipped
            // and its outputs are NaN, the loud failure of a mismatched shape.
            for (int64_t e = t; e < 6 * (S + 1); e += kThreads) out[e] = __longlong_as_double(0x7ff8000000000000LL);
            __syncthreads();
            continue;
        }

        if (t == 0) {
            s_gate = gate_index(f, I.n_field, S, I.gate_floor);
            // PopInt window from the reference's findinterval (tools_algorithmic.c:19-43)
            const int64_t num_r = n - 1;
            int64_t lo = -1, hi;
            if (!(-G.x_int < G.x[0])) {
                int64_t i = 0;
                while (i < num_r && !(-G.x_int <= G.x[i + 1])) i++;
                lo = i;
            }
            if (G.x_int < G.x[0]) {
                hi = 0;
            } else {
                int64_t i = 0;
                while (i < num_r && !(G.x_int <= G.x[i + 1])) i++;
                hi = (i < num_r) ? i + 1 : num_r + 1;
            }
            s_lo = lo < 0 ? 0 : lo;
            s_hi = hi > num_r ? num_r : hi;
        }
        for (int64_t i = 0; i < m; i++) {
            int64_t q = i * kThreads + t;
            psi[q] = P0[q];
        }
        __syncthreads();
        const int64_t lo = s_lo, hi = s_hi, gate = s_gate;
        {   // initial window population (prop.c:87-93)
            double v[1] = {0.0};
            for (int64_t i = 0; i < m; i++) {
                int64_t j = t * m + i, q = i * kThreads + t;
                if (j >= lo && j <= hi) v[0] += psi[q].re * psi[q].re + psi[q].im * psi[q].im;
            }
            block_sum<1>(v, red);
            if (t == 0) {
                o_t[0] = I.tmin;
                o_e[0] = 0.0;
                o_src[0] = 0.0;
                o_ptot[0] = 1.0;
                o_pint[0] = v[0];
                o_x[0] = 0.0;
            }
        }
        double tt = I.tmin;
        const int64_t s0 = t * m;
        const double xs = (s0 < n) ? GVX[t].im : 0.0;
        const bool ckpt = I.ckpt_every > 0 && I.ckpt_off >= 0 && P.snapshots;
        auto store_state = [&](int64_t slot) {  // natural order, 2n doubles per slot
            double* dst = P.snapshots + I.ckpt_off + slot * 2 * n;
            for (int64_t i = 0; i < m; i++)
                if (s0 + i < n) st2(dst + 2 * (s0 + i), psi[i * kThreads + t]);
        };
        if (ckpt) store_state(0);

        for (int64_t k = 0; k < S; k++) {
            const double Fk = (k <= gate || k >= I.n_field) ? 0.0 : f[k];
            if (t == 0) {
                if (k > 0) {  // finish the previous step's observables
                    double s[5];
#pragma unroll
                    for (int c = 0; c < 5; c++) {
                        s[c] = 0.0;
#pragma unroll
                        for (int q = 0; q < kWarps; q++) s[c] += red[q * 5 + c];
                    }
                    o_src[k] = -s[0] + o_e[k];
                    o_ptot[k] = s[2] * s[2] + s[3] * s[3];
                    o_x[k] = s[1];
                    o_pint[k] = s[4];
                }
                tt += dt;
                o_t[k + 1] = tt;
                o_e[k + 1] = Fk;
            }
            double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
            cn_step_fp64(psi, yl, tab, m, L, Fk, dt, dx, xs, sc, sb, [&](int64_t q, int64_t i, const cd& pn) {
                const int64_t j = s0 + i;
                const double n2 = fma(pn.re, pn.re, pn.im * pn.im);
                const cd gx = GVX[q];
                const cd p0 = P0[q];
                acc[0] = fma(n2, gx.re, acc[0]);
                acc[1] = fma(n2, gx.im, acc[1]);
                acc[2] = fma(pn.re, p0.re, fma(pn.im, p0.im, acc[2]));
                acc[3] = fma(pn.re, p0.im, fma(-pn.im, p0.re, acc[3]));
                if (j >= lo && j <= hi) acc[4] += n2;
            });
#pragma unroll
            for (int c = 0; c < 5; c++)
#pragma unroll
                for (int d = 16; d >= 1; d >>= 1) acc[c] += shfl_xor(acc[c], d);
            if (lane == 0)
#pragma unroll
                for (int c = 0; c < 5; c++) red[w * 5 + c] = acc[c];
            if (ckpt && (k + 1) % I.ckpt_every == 0 && k + 1 < S) store_state((k + 1) / I.ckpt_every);
            if (I.snap_off >= 0 && P.snapshots) {  // prop.c:248-263
                int64_t slot = -1;
                if (k % I.snap_every == 0 && k / I.snap_every < I.n_snap - 1) slot = k / I.snap_every;
                if (k == S - 1) slot = I.n_snap - 1;
                if (slot >= 0) {
                    double* sp = P.snapshots + I.snap_off + slot * 2 * n;
                    for (int64_t i = 0; i < m; i++) {
                        int64_t j = s0 + i;
                        if (j < n) st2(sp + 2 * j, psi[i * kThreads + t]);
                    }
                }
            }
            __syncthreads();
        }
        if (t == 0) {
            double s[5];
#pragma unroll
            for (int c = 0; c < 5; c++) {
                s[c] = 0.0;
#pragma unroll
                for (int q = 0; q < kWarps; q++) s[c] += red[q * 5 + c];
            }
            o_src[S] = -s[0] + o_e[S];
            o_ptot[S] = s[2] * s[2] + s[3] * s[3];
            o_x[S] = s[1];
            o_pint[S] = s[4];
        }
        if (P.psi_final && I.psi_off >= 0) {
            double* pf = P.psi_final + I.psi_off;
            for (int64_t i = 0; i < m; i++) {
                int64_t j = s0 + i;
                if (j < n) st2(pf + 2 * j, psi[i * kThreads + t]);
            }
        }
        __syncthreads();
    }
}

}  // namespace mma

using namespace mma;

// ------------------------------------------------------------------------------------------
// Host entry points of the batched surface.
// ------------------------------------------------------------------------------------------
extern "C" int mma_tdse_build_grids(const mma_tdse_grid* grids_dev, const mma_tdse_grid* grids_host, int n_grids,
                                    int mode, void* stream)
{
    if (n_grids <= 0 || !grids_dev || !grids_host || (mode != 0 && mode != 1)) return MMA_ERR_ARG;
    for (int g = 0; g < n_grids; g++) {
        const mma_tdse_grid& G = grids_host[g];
        if (G.n < 3 || G.m < 1 || G.m * kThreads < G.n || !(G.dx > 0.0) || !(G.dt > 0.0) || !G.x || !G.gv ||
            !G.psi0 || !G.cn_tab || !G.gs_tab || !G.result || !(G.trg_a == G.trg_a))
            return MMA_ERR_ARG;
        if (mode == 0 && G.max_iter < 1) return MMA_ERR_ARG;
    }
    build_grids_kernel<<<n_grids, kThreads, 0, (cudaStream_t)stream>>>(grids_dev, mode);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

static bool psi_fits_smem(int max_m) { return (size_t)max_m * kThreads * 16 <= 220 * 1024; }

static int sm_count()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

extern "C" int mma_tdse_propagate_c64_impl(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                           const mma_tdse_buffers* bufs, int m32, int cta_threads, int grid_ctas,
                                           void* stream);

extern "C" int mma_tdse_propagate_df64_impl(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                            const mma_tdse_buffers* bufs, int max_m, int grid_ctas, void* stream);
extern "C" int mma_tdse_df64_default_ctas();
extern "C" int mma_tdse_c64_default_ctas(int m32, int cta_threads);
extern "C" size_t mma_tdse_df64_scratch_bytes(int max_m, int grid_ctas);

extern "C" int mma_tdse_default_ctas(int max_m, int precision)
{
    const int sms = sm_count();
    if (sms <= 0 || max_m < 1) return 0;
    if (precision == 1) {  // complex64 form with 256-thread tables of m32 = max_m sites per thread
        const int c = mma_tdse_c64_default_ctas(max_m, 0);
        return c > 0 ? c : sms;
    }
    if (precision == 2) return mma_tdse_df64_default_ctas();
    int per_sm = 1;
    if (psi_fits_smem(max_m)) {
        size_t smem = (size_t)max_m * kThreads * 16;
        cudaFuncSetAttribute(propagate_fp64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, propagate_fp64_kernel<true>, kThreads, smem);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, propagate_fp64_kernel<false>, kThreads, 0);
    }
    return sms * (per_sm > 0 ? per_sm : 1);
}

extern "C" size_t mma_tdse_scratch_bytes(int max_m, int grid_ctas, int precision)
{
    if (precision == 1) return 8;  // complex64 form keeps its sweep in registers
    if (grid_ctas <= 0) grid_ctas = mma_tdse_default_ctas(max_m, precision);
    if (grid_ctas <= 0) grid_ctas = 1;
    if (precision == 2) return mma_tdse_df64_scratch_bytes(max_m, grid_ctas);
    size_t per = (size_t)max_m * kThreads * 16;
    return per * (size_t)grid_ctas * (psi_fits_smem(max_m) ? 1 : 2);
}

extern "C" int mma_tdse_propagate(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                  const mma_tdse_buffers* bufs, int max_m, int grid_ctas, int precision, void* stream)
{
    return mma_tdse_propagate_ex(insts, n_inst, grids, bufs, max_m, 0, grid_ctas, precision, stream);
}

extern "C" int mma_tdse_propagate_ex(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                     const mma_tdse_buffers* bufs, int max_m, int cta_threads, int grid_ctas,
                                     int precision, void* stream)
{
    if (n_inst <= 0) return MMA_OK;
    if (precision < 0 || precision > 2) return MMA_ERR_UNSUPPORTED;
    // max_m = 0 is the complex64 form's "every 256-thread table width" launch
    if (!insts || !grids || !bufs || !bufs->fields || !bufs->outputs || !bufs->counter || !bufs->scratch ||
        max_m < (precision == 1 ? 0 : 1))
        return MMA_ERR_ARG;
    if (sm_count() <= 0) return MMA_ERR_NO_DEVICE;
    if (grid_ctas <= 0)
        grid_ctas = precision == 1 ? mma_tdse_c64_default_ctas(max_m, cta_threads) : mma_tdse_default_ctas(max_m, precision);
    if (grid_ctas <= 0) return MMA_ERR_TOO_LARGE;  // no complex64 kernel for this shape
    if (grid_ctas > n_inst) grid_ctas = n_inst;
    if (precision == 1) {
        // max_m is the common m32 of the batch's complex64 tables, cta_threads their CTA size
        return mma_tdse_propagate_c64_impl(insts, n_inst, grids, bufs, max_m, cta_threads, grid_ctas, stream);
    }
    if (cta_threads != 0 && cta_threads != kThreads) return MMA_ERR_UNSUPPORTED;
    if (bufs->scratch_bytes < mma_tdse_scratch_bytes(max_m, grid_ctas, precision)) return MMA_ERR_ARG;
    if (precision == 2)  // float-float form: the FP64 layout, psi in scratch, two CTAs per SM
        return mma_tdse_propagate_df64_impl(insts, n_inst, grids, bufs, max_m, grid_ctas, stream);
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(bufs->counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    PropArgs A{insts, n_inst, grids, bufs->fields, bufs->outputs, bufs->psi_final, bufs->snapshots, bufs->counter,
               (double*)bufs->scratch, (int64_t)max_m * kThreads};
    if (psi_fits_smem(max_m)) {
        size_t smem = (size_t)max_m * kThreads * 16;
        cudaFuncSetAttribute(propagate_fp64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        propagate_fp64_kernel<true><<<grid_ctas, kThreads, smem, st>>>(A);
    } else {
        propagate_fp64_kernel<false><<<grid_ctas, kThreads, 0, st>>>(A);
    }
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

// ------------------------------------------------------------------------------------------
// Allocation-free propagation.
//
// For callers that cannot allocate device memory themselves -- a host embedded in a
// process whose device memory belongs to another runtime's pool (a framework caching
// allocator with a hard cap, a plugin host that hands out only the buffers it owns),
// or code that must not allocate while a graph is being recorded -- this entry point
// runs the same FP64 propagation kernel with its work space (the work-queue counter and
// the per-CTA sweep buffer) taken from a fixed array compiled into this library instead
// of a caller-provided scratch buffer.  The caller still passes inputs and outputs.
// ------------------------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr size_t kNoAllocBytes = (size_t)8 << 20;  // 8 MiB on every device that loads the library
constexpr size_t kNoAllocHeader = 256;            // work-queue counter lives in the first 256 bytes
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

// Device address of g_noalloc_scratch on the current device.  The symbol's host-side name
// is only a stand-in, so the address is looked up once per device, with that device current.
int noalloc_address(void** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MMA_ERR_NO_DEVICE;
    if (dev < 0 || dev >= 64) return MMA_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MMA_ERR_CUDA;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return MMA_OK;
}

}  // namespace

extern "C" size_t mma_tdse_noalloc_capacity_bytes(void) { return kNoAllocBytes; }

extern "C" int mma_tdse_propagate_noalloc(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                          const double* fields, double* outputs, double* psi_final,
                                          double* snapshots, int max_m, void* stream)
{
    if (n_inst <= 0) return MMA_OK;
    if (!insts || !grids || !fields || !outputs || max_m < 1) return MMA_ERR_ARG;
    // one CTA needs max_m * 256 * 16 bytes of sweep buffer, and the wavefunction must fit
    // in shared memory (the fixed array does not also hold it)
    const size_t per_cta = (size_t)max_m * kThreads * 16;
    if (!psi_fits_smem(max_m) || per_cta > kNoAllocBytes - kNoAllocHeader) return MMA_ERR_TOO_LARGE;
    if (sm_count() <= 0) return MMA_ERR_NO_DEVICE;
    void* base = nullptr;
    int rc = noalloc_address(&base);
    if (rc != MMA_OK) return rc;
    int ctas = mma_tdse_default_ctas(max_m, 0);
    const int cap = (int)((kNoAllocBytes - kNoAllocHeader) / per_cta);
    if (ctas > cap) ctas = cap;
    if (ctas > n_inst) ctas = n_inst;
    if (ctas < 1) return MMA_ERR_TOO_LARGE;
    cudaStream_t st = (cudaStream_t)stream;
    int* counter = reinterpret_cast<int*>(base);
    // the array keeps the previous call's contents: the work-queue head must restart at 0
    if (cudaMemsetAsync(counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    PropArgs A{insts, n_inst, grids, fields, outputs, psi_final, snapshots, counter,
               reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kNoAllocHeader),
               (int64_t)max_m * kThreads};
    const size_t smem = per_cta;
    cudaFuncSetAttribute(propagate_fp64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    propagate_fp64_kernel<true><<<ctas, kThreads, smem, st>>>(A);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
