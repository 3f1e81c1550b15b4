// tdse_step.cuh -- table layout and one FP64 Crank-Nicolson-Numerov step, shared by the
// propagation kernel and the adjoint kernel's forward recompute.
#pragma once

#include "common.cuh"
#include "tdse_solver.cuh"

namespace mma {

// Slots of the complex CN table (each L = m*kThreads complex entries, chunk-interleaved).
enum { CN_IB6 = 0, CN_H, CN_F, CN_G, CN_GG, CN_PSI0, CN_GVX, CN_SLOTS };
// Slots of the real ground-state table.
enum { GS_IB12 = 0, GS_H, GS_F, GS_G, GS_GG, GS_SLOTS };
// Slots of the adjoint (A^H) table: the first five CN slots.
constexpr int ADJ_SLOTS = 5;

__device__ __forceinline__ double soft_coulomb(double x, double a) { return -1.0 / sqrt(a * a + x * x); }
__device__ __forceinline__ double minus_grad_v(double x, double a) { return x * pow(a * a + x * x, -1.5); }

__device__ __forceinline__ int64_t qidx(int64_t j, int64_t m) { return (j % m) * kThreads + (j / m); }

// First index where the reference's zero gate opens: the first k with f[k] f[k+1] <= 0
// (prop.c:125-134); samples at and beyond n_field are zero, and samples with
// |f| <= floor count as zero in this test (floor is 0 unless the field was
// Fourier-interpolated, where it absorbs the transform's round-off).
__device__ inline int64_t gate_index(const double* f, int64_t n_field, int64_t n_steps, double floor_)
{
    for (int64_t k = 0; k < n_steps; k++) {
        double a = (k < n_field) ? f[k] : 0.0, b = (k + 1 < n_field) ? f[k + 1] : 0.0;
        if (fabs(a) <= floor_) a = 0.0;
        if (fabs(b) <= floor_) b = 0.0;
        if (a * b <= 0.0) return k;
    }
    return n_steps;
}

// One step psi <- e^{+i F dt x} (A^{-1}(2 M2 psi) - psi) on a chunk-interleaved vector
// (shared or global memory), tables `tab` of one grid (tdse_solver.cuh describes the
// partitioned solve).  obs(q, i, psi_new) is called for every site of the thread's chunk
// in the last pass.  Contains the scans' two __syncthreads.
template <typename Obs>
__device__ __forceinline__ void cn_step_fp64(cd* psi, cd* yl, const cd* tab, int64_t m, int64_t L, double Fk,
                                             double dt, double dx, double xs, cd* sc, cd* sb, Obs obs)
{
    const int t = threadIdx.x;
    const cd *ib6 = tab + CN_IB6 * L, *hh = tab + CN_H * L, *FF = tab + CN_F * L, *gg = tab + CN_G * L,
             *GG = tab + CN_GG * L;
    // ---- pass 1: local forward sweep of the right-hand side 2 M2 psi
    cd pm = (t == 0) ? cd{0.0, 0.0} : psi[(m - 1) * kThreads + t - 1];
    cd pc = psi[t];
    cd yprev{0.0, 0.0};
    for (int64_t i = 0; i < m; i++) {
        int64_t q = i * kThreads + t;
        cd pn = (i + 1 < m) ? psi[q + kThreads] : ((t + 1 < kThreads) ? psi[t + 1] : cd{0.0, 0.0});
        cd r{fma(10.0, pc.re, pm.re + pn.re), fma(10.0, pc.im, pm.im + pn.im)};
        cd y = cfms(hh[q], yprev, cmul(ib6[q], r));
        yl[q] = y;
        yprev = y;
        pm = pc;
        pc = pn;
    }
    const cd yin = scan_forward<cd>(FF[(m - 1) * kThreads + t], yprev, sc, sb);
    // ---- pass 2: local backward sweep with the forward correction
    cd unext{0.0, 0.0};
    for (int64_t i = m - 1; i >= 0; i--) {
        int64_t q = i * kThreads + t;
        cd y = cfma(FF[q], yin, yl[q]);
        cd u = cfms(gg[q], unext, y);
        yl[q] = u;
        unext = u;
    }
    const cd uin = scan_backward<cd>(GG[t], unext, sc + kWarps, sb + kWarps);
    // ---- pass 3: backward correction, CN update, phase e^{+i F dt x}
    double sn, cs;
    sincos(Fk * dt * xs, &sn, &cs);
    cd ph{cs, sn};
    sincos(Fk * dt * dx, &sn, &cs);
    const cd z{cs, sn};
    for (int64_t i = 0; i < m; i++) {
        int64_t q = i * kThreads + t;
        cd u = cfma(GG[q], uin, yl[q]);
        cd d = u - psi[q];
        cd pn = cmul(ph, d);
        psi[q] = pn;
        ph = cmul(ph, z);
        obs(q, i, pn);
    }
}

}  // namespace mma
