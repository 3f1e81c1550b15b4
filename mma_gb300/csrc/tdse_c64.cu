// tdse_c64.cu -- complex64 form of the TDSE propagation (the precision-chosen form).
//
// Same Crank-Nicolson-Numerov step and the same partitioned solve as the FP64 kernel
// (tdse_kernels.cu, tdse_solver.cuh), with:
//   * the factorisation computed in FP64 (build_grids_kernel) and rounded once to FP32;
//   * the wavefunction and the sweep in FP32 registers: each of the 256 threads keeps its
//     M <= 48 sites of psi and of the sweep in registers for the whole pulse.  Instead of
//     storing the chunk products of the partitioned solve, each sweep is run twice: once
//     from zero to get the chunk-boundary carry for the CTA scan, once from the exact carry
//     (five passes per step, registers 4M floats);
//   * the per-site tables in shared memory, 16 bytes per site: 1/(2 beta) (complex), V_j and the
//     (real) ground state.  h_j = 6 a_j/beta_j and g_j = 6 c_j/beta_j are re-derived from
//     1/(2 beta) and w_q = dt/2 (-1/(2dx^2) + V_q/12) (a_j = 1/12 + i w_{j-1}, c_j = 1/12 + i w_{j+1}),
//     and -V'_j = -x_j V_j^3 -- nothing per step goes to L2 but the four observables.  Storing
//     half of 1/beta (a power of two, so no rounding changes) halves y and u throughout the
//     solve and saves the multiplications by 1/2 in h and g; the update takes 2u - psi;
//   * the phase e^{+i E dt x}: the chunk-start angle is formed and reduced mod 2 pi in
//     float-float arithmetic, then e^{i E dt dx i} per site from a table;
//   * the observables summed per thread with Kahan compensation, across the warp with
//     two-sum pairs, across warps with two-sum pairs by warp 0;
//   * no serial FP64 on single warps (a 32-lane FP64 instruction holds a sub-partition's FP64
//     unit for about 64 cycles, and a late warp stalls the others at the next scan barrier):
//     the field-derived tables are filled for a block of steps by all warps, one step each, and
//     the observables are converted to FP64 once per block, one step per lane.
// Reference: 1DTDSE/sources/prop.c:115-347 (step and observables), tridiag.c:26-70 (solve).
#include <cuda_runtime.h>

#include "../../include/mma_tdse.h"
#include "common.cuh"

namespace mma {
namespace c64 {

struct cf {
    float re, im;
};
__device__ __forceinline__ cf operator+(cf a, cf b) { return cf{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf operator-(cf a, cf b) { return cf{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cf cmul(cf a, cf b) { return cf{fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re)}; }
// a + b*c
__device__ __forceinline__ cf cfma(cf b, cf c, cf a)
{
    return cf{fmaf(b.re, c.re, fmaf(-b.im, c.im, a.re)), fmaf(b.re, c.im, fmaf(b.im, c.re, a.im))};
}
// a - b*c
__device__ __forceinline__ cf cfms(cf b, cf c, cf a)
{
    return cf{fmaf(-b.re, c.re, fmaf(b.im, c.im, a.re)), fmaf(-b.re, c.im, fmaf(-b.im, c.re, a.im))};
}
__device__ __forceinline__ cf shup(cf v, int d)
{
    return cf{__shfl_up_sync(0xffffffffu, v.re, d), __shfl_up_sync(0xffffffffu, v.im, d)};
}
__device__ __forceinline__ cf shdn(cf v, int d)
{
    return cf{__shfl_down_sync(0xffffffffu, v.re, d), __shfl_down_sync(0xffffffffu, v.im, d)};
}

// Table slots (floats), each L = 256*M long, site j = t*M + i at q = i*256 + t.
enum { T_IBRE = 0, T_IBIM, T_V, T_PSI0, T_SLOTS };

// forward scan of Y_t = b_t + c_t Y_{t-1} over the CTA of NW warps, exclusive (see tdse_solver.cuh)
template <int NW = kWarps>
__device__ __forceinline__ cf scan_fwd(cf c, cf b, cf* sc, cf* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        cf cp = shup(c, d), bp = shup(b, d);
        if (lane >= d) {
            b = cfma(c, bp, b);
            c = cmul(c, cp);
        }
    }
    if (lane == 31) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    cf yw{0.f, 0.f};
    for (int q = 0; q < NW; q++)
        if (q < w) yw = cfma(sc[q], yw, sb[q]);
    cf cp = shup(c, 1), bp = shup(b, 1);
    return lane == 0 ? yw : cfma(cp, yw, bp);
}

template <int NW = kWarps>
__device__ __forceinline__ cf scan_bwd(cf c, cf b, cf* sc, cf* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        cf cp = shdn(c, d), bp = shdn(b, d);
        if (lane + d < 32) {
            b = cfma(c, bp, b);
            c = cmul(c, cp);
        }
    }
    if (lane == 0) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    cf uw{0.f, 0.f};
    for (int q = NW - 1; q >= 0; q--)
        if (q > w) uw = cfma(sc[q], uw, sb[q]);
    cf cp = shdn(c, 1), bp = shdn(b, 1);
    return lane == 31 ? uw : cfma(cp, uw, bp);
}


// error-free sum (Knuth two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

struct Args {
    const mma_tdse_instance* insts;
    int n_inst;
    const mma_tdse_grid* grids;
    const double* fields;
    double* outputs;
    double* psi_final;
    double* snapshots;
    int* counter;
};

// First index where the zero gate opens (prop.c:125-134), as in the FP64 kernel.
__device__ int64_t gate_index32(const double* f, int64_t n_field, int64_t n_steps, double floor_)
{
    for (int64_t k = 0; k < n_steps; k++) {
        double a = (k < n_field) ? f[k] : 0.0, b = (k + 1 < n_field) ? f[k + 1] : 0.0;
        if (fabs(a) <= floor_) a = 0.0;
        if (fabs(b) <= floor_) b = 0.0;
        if (a * b <= 0.0) return k;
    }
    return n_steps;
}

constexpr double kInvTwoPi = 0.15915494309189533576888376337251;

// Outputs of an instance whose grid has no tables of the launched shape: NaN (a loud failure).
__device__ __forceinline__ void nan_outputs(const Args& P, const mma_tdse_instance& I, int T)
{
    for (int64_t q = threadIdx.x; q < 6 * (I.n_steps + 1); q += T)
        P.outputs[I.out_off + q] = __longlong_as_double(0x7ff8000000000000LL);
    __syncthreads();
}


// The grid whose tables a CTA holds in shared memory (-1: none yet), common to every width.
__shared__ int64_t c64_s_grid;

// One instance of the register-resident form (T = 256 threads, M sites per thread): the
// instance's tables are loaded into tab4 unless c64_s_grid says they are there already.
template <int M>
__device__ __forceinline__ void c64_reg_instance(const Args& P, const mma_tdse_instance& I, const mma_tdse_grid& G)
{
    extern __shared__ float4 tab4[];  // the kernel's dynamic shared memory (named here: shared loads)
    int64_t& s_grid = c64_s_grid;
    __shared__ cf sc[2 * kWarps], sb[2 * kWarps];
    __shared__ float red_hi[kWarps * 4], red_lo[kWarps * 4];
    __shared__ cf bfirst[kWarps], blast[kWarps];
    // field-derived tables for a block of KB = kWarps steps, filled at the block's first step with
    // one step per warp: e^{i F_k dt dx i} (i < M: phase of site i relative to site 0) and F_k dt
    // as a float-float pair (phase angle of pass 5)
    constexpr int KB = kWarps;
    __shared__ cf s_wtab[KB][M];
    __shared__ float s_ahi[KB], s_alo[KB];
    __shared__ float obs_h[KB][4], obs_l[KB][4];  // observables' totals, FP64 once per KB steps
    __shared__ int64_t s_gate, s_lo, s_hi;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    constexpr int L = kThreads * M;
    const int64_t n = G.n, S = I.n_steps;
    // ---- tables into shared memory when the grid changes
    if (s_grid != I.grid) {
        for (int q = t; q < L; q += kThreads)
            tab4[q] = make_float4(G.c64_tab[T_IBRE * L + q], G.c64_tab[T_IBIM * L + q], G.c64_tab[T_V * L + q],
                                  G.c64_tab[T_PSI0 * L + q]);
    }
    __syncthreads();
    if (t == 0) {
        s_grid = I.grid;
        s_gate = gate_index32(P.fields + I.field_off, I.n_field, S, I.gate_floor);
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
    // ---- state: psi in registers, initialised from the ground state
    cf psi[M], yy[M];
    const int64_t s0 = (int64_t)t * M;
#pragma unroll
    for (int i = 0; i < M; i++) psi[i] = cf{tab4[i * kThreads + t].w, 0.f};
    // chunk start x as a float-float pair (phase angle) and as a float (<x>, -V')
    const double xs_d = (s0 < n) ? G.x[s0] : 0.0;
    const float xs_hi = (float)xs_d, xs_lo = (float)(xs_d - (double)xs_hi);
    const float dxf = (float)G.dx;
    const double dt = G.dt;
    // 6 w_q = 6 dt/2 (-1/(2 dx^2)) + (dt/4) V_q.  The constant is carried as a float-float
    // pair (c_hi + c_lo): rounded once to float it would be the same error at every site,
    // a slightly different kinetic scale whose phase error grows step after step.
    const double c6 = 6.0 * 0.5 * dt * (-0.5 / (G.dx * G.dx));
    const float c_hi = (float)c6, c_lo = (float)(c6 - (double)c_hi), c1 = (float)(0.25 * dt);
    if (lane == 0) bfirst[w] = psi[0];
    if (lane == 31) blast[w] = psi[M - 1];
    __syncthreads();
    const int64_t lo = s_lo, hi = s_hi, gate = s_gate;
    // this thread's part of the population window [lo, hi], as chunk indices
    const int win_a = (int)max((int64_t)0, lo - s0), win_b = (int)min((int64_t)M - 1, hi - s0);
    const double* f = P.fields + I.field_off;
    double* out = P.outputs + I.out_off;
    double *o_t = out, *o_e = out + (S + 1), *o_src = out + 2 * (S + 1), *o_ptot = out + 3 * (S + 1),
           *o_pint = out + 4 * (S + 1), *o_x = out + 5 * (S + 1);
    {   // initial window population (prop.c:87-93), FP64 from the FP64 ground state
        double v[1] = {0.0};
        for (int64_t j = t; j < n; j += kThreads)
            if (j >= lo && j <= hi) v[0] += G.psi0[2 * j] * G.psi0[2 * j] + G.psi0[2 * j + 1] * G.psi0[2 * j + 1];
        block_sum<1>(v, reinterpret_cast<double*>(red_hi));
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
    // h_j and g_j of site (i, t): 6 a_j /beta_j and 6 c_j /beta_j from the neighbour's V,
    // (1 + i 12 w) * ib2 with ib2 = 1/(2 beta) (the table) and 12 w = c_hi2 + (c_lo2 + c12 V)
    // kept unsummed -- bit for bit (1/2 + i 6 w) / beta, every factor being scaled by 2.  No
    // boundary tests: rows beyond n-1 have zero tables (y = u = 0 there), the first row's h
    // multiplies an incoming carry of 0 and the last row's g multiplies u_n = 0.
    const float c_hi2 = 2.f * c_hi, c_lo2 = 2.f * c_lo, c12 = 2.f * c1;
    auto off_diag = [&](float v, float ir, float ii) -> cf {
        const float t1 = fmaf(c12, v, c_lo2);
        return cf{fmaf(-t1, ii, fmaf(-c_hi2, ii, ir)), fmaf(t1, ir, fmaf(c_hi2, ir, ii))};
    };
    const float v_left = (t == 0) ? 0.f : tab4[(M - 1) * kThreads + t - 1].z;   // V left of site 0
    const float v_right = (t == kThreads - 1) ? 0.f : tab4[t + 1].z;            // V right of site M-1

    // observables of output index ko (the state after step ko - 1), warp 0: lanes 8c+q hold
    // warp q's two-sum pair of observable c; reduced over q into ring slot (ko - 1) mod KB
    auto obs_reduce = [&](int64_t ko) {
        const int c = lane >> 3, q = lane & 7;
        float hs = red_hi[q * 4 + c], ls = red_lo[q * 4 + c];
#pragma unroll
        for (int d = 4; d >= 1; d >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hs, d);
            const float ol = __shfl_xor_sync(0xffffffffu, ls, d);
            float s2, e2;
            two_sum(hs, oh, s2, e2);
            hs = s2;
            ls += ol + e2;
        }
        if (q == 0) {
            const int j = (int)((ko - 1) % KB);
            obs_h[j][c] = hs;
            obs_l[j][c] = ls;
        }
    };
    // FP64 outputs of the cnt indices ending at k_last, one per lane: sourceterm -<V'> + F of
    // the step before, <x> and |<psi0|psi>|^2 (prop.c:266-300)
    auto obs_flush = [&](int64_t k_last, int cnt) {
        __syncwarp();
        if (lane < cnt) {
            const int64_t ko = k_last - cnt + 1 + lane, kp = ko - 1;
            const int j = (int)(kp % KB);
            double v[4];
#pragma unroll
            for (int c = 0; c < 4; c++) v[c] = (double)obs_h[j][c] + (double)obs_l[j][c];
            o_src[ko] = -v[0] + ((kp <= gate || kp >= I.n_field) ? 0.0 : __ldg(f + kp));
            o_x[ko] = v[1];
            o_ptot[ko] = fma(v[2], v[2], v[3] * v[3]);
        }
        __syncwarp();
    };
    for (int64_t k = 0; k < S; k++) {
        // FP64 work is kept off single warps (a 32-lane FP64 instruction holds a sub-partition's
        // FP64 unit for about 64 cycles): warp 0 reduces the previous step's observables in FP32
        // and converts them once per KB steps, one step per lane; the field tables are filled
        // once per KB steps by all warps; warp 1 lane 0 advances the time grid.
        if (w == 0 && k > 0) {
            obs_reduce(k);
            if ((k - 1) % KB == KB - 1) obs_flush(k, KB);
        }
        if (w == 1 && lane == 0) {
            tt += dt;
            o_t[k + 1] = tt;
            o_e[k + 1] = (k <= gate || k >= I.n_field) ? 0.0 : __ldg(f + k);
        }
        if (k % KB == 0) {
            // per-site phase factors of step k + w, each from its own angle: a recurrence in i
            // would carry the FP32 rounding of |e^{i F dt dx}| (1 +- 6e-8) as a bias growing
            // with i, and it would compound over the steps into a drift of the norm along each
            // chunk.  Read in pass 5, after the scans' barriers; refilled after the end-of-step
            // barrier of the block's last step.
            const int64_t ks = k + w;
            const double Fs = (ks <= gate || ks >= I.n_field || ks >= S) ? 0.0 : __ldg(f + ks);
            for (int i = lane; i < M; i += 32) {
                float sn, cs;
                sincosf((float)(Fs * dt * G.dx) * (float)i, &sn, &cs);
                s_wtab[w][i] = cf{cs, sn};
            }
            if (lane == 0) {
                const double fdt = Fs * dt;
                const float a_hi = (float)fdt;
                s_ahi[w] = a_hi;
                s_alo[w] = (float)(fdt - (double)a_hi);
            }
        }
        // right-hand side 2 M2 psi at site i (neighbours across threads by shuffle/shared)
        cf left = shup(psi[M - 1], 1), right = shdn(psi[0], 1);
        if (lane == 0) left = (w == 0) ? cf{0.f, 0.f} : blast[w - 1];
        if (lane == 31) right = (w == kWarps - 1) ? cf{0.f, 0.f} : bfirst[w + 1];
        // ---- pass 1: local forward sweep from zero: chunk-end value and product of (-h)
        cf yprev{0.f, 0.f}, Fp{1.f, 0.f};
        float vl = v_left;
#pragma unroll
        for (int i = 0; i < M; i++) {
            const float4 tb = tab4[i * kThreads + t];
            const cf pm = (i == 0) ? left : psi[i - 1];
            const cf pn = (i == M - 1) ? right : psi[i + 1];
            const cf r{fmaf(10.f, psi[i].re, pm.re + pn.re), fmaf(10.f, psi[i].im, pm.im + pn.im)};
            const cf h = off_diag(vl, tb.x, tb.y);
            yprev = cfms(h, yprev, cmul(cf{tb.x, tb.y}, r));
            Fp = cmul(Fp, cf{-h.re, -h.im});
            vl = tb.z;
        }
        cf yc = scan_fwd(Fp, yprev, sc, sb);  // exact y at the end of the previous chunk
        // ---- pass 2: forward sweep again from the exact carry, kept in registers
        vl = v_left;
#pragma unroll
        for (int i = 0; i < M; i++) {
            const float4 tb = tab4[i * kThreads + t];
            const cf pm = (i == 0) ? left : psi[i - 1];
            const cf pn = (i == M - 1) ? right : psi[i + 1];
            const cf r{fmaf(10.f, psi[i].re, pm.re + pn.re), fmaf(10.f, psi[i].im, pm.im + pn.im)};
            yc = cfms(off_diag(vl, tb.x, tb.y), yc, cmul(cf{tb.x, tb.y}, r));
            yy[i] = yc;
            vl = tb.z;
        }
        // ---- pass 3: local backward sweep from zero: chunk-start value and product of (-g)
        cf unext{0.f, 0.f}, Gp{1.f, 0.f};
        float vr = v_right;
#pragma unroll
        for (int i = M - 1; i >= 0; i--) {
            const float4 tb = tab4[i * kThreads + t];
            const cf g = off_diag(vr, tb.x, tb.y);
            unext = cfms(g, unext, yy[i]);
            Gp = cmul(Gp, cf{-g.re, -g.im});
            vr = tb.z;
        }
        cf uc = scan_bwd(Gp, unext, sc + kWarps, sb + kWarps);  // exact u at the start of the next chunk
        // ---- pass 4: backward sweep again from the exact carry
        vr = v_right;
#pragma unroll
        for (int i = M - 1; i >= 0; i--) {
            const float4 tb = tab4[i * kThreads + t];
            uc = cfms(off_diag(vr, tb.x, tb.y), uc, yy[i]);
            yy[i] = uc;
            vr = tb.z;
        }
        // ---- pass 5: CN update, phase, observables
        // chunk-start angle F dt x_s in float-float, reduced mod 2 pi
        const int kb = (int)(k % KB);
        const float a_hi = s_ahi[kb], a_lo = s_alo[kb];
        float th_hi = a_hi * xs_hi;
        float th_lo = fmaf(a_hi, xs_hi, -th_hi) + fmaf(a_hi, xs_lo, a_lo * xs_hi);
        const float kk = rintf(th_hi * (float)kInvTwoPi);
        // 2 pi = C1 + C2 + C3 (C1, C2 exact in float)
        const float C1 = 6.28125f, C2 = 1.93500518798828125e-3f, C3 = 3.0199159819370158e-07f;
        float red = fmaf(-kk, C1, th_hi);
        red = fmaf(-kk, C2, red);
        red = fmaf(-kk, C3, red) + th_lo;
        float sn, cs;
        sincosf(red, &sn, &cs);
        const cf phs{cs, sn};
        // compensated sums: FP32 blocks of 16 sites, then an error-free update of (hi, lo)
        float acc_hi[4] = {0.f, 0.f, 0.f, 0.f}, acc_lo[4] = {0.f, 0.f, 0.f, 0.f}, part[4] = {0.f, 0.f, 0.f, 0.f};
        float pint = 0.f;
#pragma unroll
        for (int i = 0; i < M; i++) {
            const float4 tb = tab4[i * kThreads + t];
            const cf d{fmaf(2.f, yy[i].re, -psi[i].re), fmaf(2.f, yy[i].im, -psi[i].im)};  // u = 2 yy
            const cf pn = cmul(cmul(phs, s_wtab[kb][i]), d);
            psi[i] = pn;
            const float n2 = fmaf(pn.re, pn.re, pn.im * pn.im);
            const float xj = fmaf(dxf, (float)i, xs_hi);
            const float vj = tb.z, pj = tb.w;
            part[0] = fmaf(n2, -xj * vj * vj * vj, part[0]);  // -V' = x (a^2+x^2)^-3/2 = -x V^3
            part[1] = fmaf(n2, xj, part[1]);
            part[2] = fmaf(pn.re, pj, part[2]);
            part[3] = fmaf(-pn.im, pj, part[3]);
            if ((i & 15) == 15 || i == M - 1) {
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    float s2, e2;
                    two_sum(acc_hi[c], part[c], s2, e2);
                    acc_hi[c] = s2;
                    acc_lo[c] += e2;
                    part[c] = 0.f;
                }
            }
            if (i >= win_a && i <= win_b) pint += n2;
        }
        if (lane == 0) bfirst[w] = psi[0];
        if (lane == 31) blast[w] = psi[M - 1];
        // warp reduction in two-sum pairs
        float hs[4], ls[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            hs[c] = acc_hi[c];
            ls[c] = acc_lo[c];
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float oh = __shfl_xor_sync(0xffffffffu, hs[c], d);
                const float ol = __shfl_xor_sync(0xffffffffu, ls[c], d);
                float s, e;
                two_sum(hs[c], oh, s, e);
                hs[c] = s;
                ls[c] += ol + e;
            }
        // the window population covers a handful of sites: plain float, FP64 across warps
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) pint += __shfl_xor_sync(0xffffffffu, pint, d);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                red_hi[w * 4 + c] = hs[c];
                red_lo[w * 4 + c] = ls[c];
            }
            sc[2 * kWarps - 1 - w].re = pint;  // parked in an idle scan slot until step end
        }
        if (I.snap_off >= 0 && P.snapshots) {  // prop.c:248-263
            int64_t slot = -1;
            if (k % I.snap_every == 0 && k / I.snap_every < I.n_snap - 1) slot = k / I.snap_every;
            if (k == S - 1) slot = I.n_snap - 1;
            if (slot >= 0) {
                double* sp = P.snapshots + I.snap_off + slot * 2 * n;
#pragma unroll
                for (int i = 0; i < M; i++)
                    if (s0 + i < n) {
                        sp[2 * (s0 + i)] = psi[i].re;
                        sp[2 * (s0 + i) + 1] = psi[i].im;
                    }
            }
        }
        __syncthreads();
        if (w == 2 && lane == 0) {
            float pi_sum = 0.f;
            for (int q = 0; q < kWarps; q++) pi_sum += sc[2 * kWarps - 1 - q].re;
            o_pint[k + 1] = (double)pi_sum;
        }
    }
    if (w == 0 && S > 0) {  // observables of the last step, then the steps not yet converted
        obs_reduce(S);
        obs_flush(S, (int)((S - 1) % KB) + 1);
    }
    if (P.psi_final && I.psi_off >= 0) {
        double* pf = P.psi_final + I.psi_off;
#pragma unroll
        for (int i = 0; i < M; i++)
            if (s0 + i < n) {
                pf[2 * (s0 + i)] = psi[i].re;
                pf[2 * (s0 + i) + 1] = psi[i].im;
            }
    }
    __syncthreads();
}

template <int M>
__global__ void __launch_bounds__(kThreads, 1) propagate_c64_kernel(Args P)
{
    __shared__ int64_t s_inst;  // tables: 256 * M sites x (1/beta re, im, V, psi0) in dynamic shared memory
    const int t = threadIdx.x;
    if (t == 0) c64_s_grid = -1;
    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        if (G.m32 != M || (G.c64_threads ? G.c64_threads : kThreads) != kThreads) {  // tables of another shape
            nan_outputs(P, I, kThreads);
            continue;
        }
        c64_reg_instance<M>(P, I, G);
    }
}

// Shared-memory form for T threads x M sites (T*M*24 bytes of shared memory: T = 256 with
// M <= 32, T = 512 with M <= 16, T = 1024 with M = 8): the wavefunction lives in shared memory
// next to the tables (24 bytes per site), which leaves registers for the chunk products F and
// G, so each sweep runs once (three passes per step); the population window is summed from
// shared memory by the threads whose chunk meets it; the observables use blocked two-sum
// accumulation (16 sites in FP32, then an error-free update of a float-float pair).  The CTA
// size T is chosen per grid (the tables are laid out for it); more threads per instance hide
// more latency at the price of wider scans.
//
// In shared memory the four tables are interleaved per site (one float4: 1/beta re, im, V,
// psi0), so each pass reads one vector per site; the neighbour's V for the off-diagonal factor
// is carried from the previous iteration.  Rows beyond n-1 have zero tables, which makes y and u
// exactly 0 there: the last row's super-diagonal then multiplies u_n = 0 and the first row's
// sub-diagonal an incoming carry of 0, so the sweeps need no boundary tests.
// One instance of the shared-memory form (T threads, M sites per thread): tables and psi in
// tab4, the tables loaded unless c64_s_grid says they are there already.
template <int M, int T>
__device__ __forceinline__ void c64_smem_instance(const Args& P, const mma_tdse_instance& I, const mma_tdse_grid& G)
{
    extern __shared__ float4 tab4[];  // the kernel's dynamic shared memory (named here: shared loads)
    int64_t& s_grid = c64_s_grid;
    constexpr int NW = T / 32;
    __shared__ cf sc[2 * NW], sb[2 * NW];
    __shared__ float red_hi[NW * 4], red_lo[NW * 4], red_pi[NW];
    // Field-derived tables for a block of KB = NW steps, filled at the block's first step with one
    // step per warp (FP64 products spread over all warps instead of one warp every step):
    // per-site phase factors e^{i F dt dx i} and F dt as a float pair.
    constexpr int KB = NW;
    __shared__ cf s_wtab[KB][M];
    __shared__ float s_ahi[KB], s_alo[KB];
    // the observables' float-pair totals of up to KB steps, converted to FP64 once per KB steps
    // across lanes (one step per lane) instead of by warp 0 every step
    __shared__ float obs_h[KB][4], obs_l[KB][4], obs_pi[KB];
    __shared__ int64_t s_gate, s_lo, s_hi;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    constexpr int L = T * M;
    cf* psi = reinterpret_cast<cf*>(tab4 + L);
    const int64_t n = G.n, S = I.n_steps;
    if (s_grid != I.grid)
        for (int q = t; q < L; q += T)
            tab4[q] = make_float4(G.c64_tab[T_IBRE * L + q], G.c64_tab[T_IBIM * L + q], G.c64_tab[T_V * L + q],
                                  G.c64_tab[T_PSI0 * L + q]);
    __syncthreads();
    if (t == 0) {
        s_grid = I.grid;
        s_gate = gate_index32(P.fields + I.field_off, I.n_field, S, I.gate_floor);
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
    const int64_t s0 = (int64_t)t * M;
#pragma unroll
    for (int i = 0; i < M; i++) psi[i * T + t] = cf{tab4[i * T + t].w, 0.f};
    const double xs_d = (s0 < n) ? G.x[s0] : 0.0;
    const float xs_hi = (float)xs_d, xs_lo = (float)(xs_d - (double)xs_hi);
    const float dxf = (float)G.dx;
    const double dt = G.dt;
    const double c6 = 6.0 * 0.5 * dt * (-0.5 / (G.dx * G.dx));
    const float c_hi = (float)c6, c_lo = (float)(c6 - (double)c_hi), c1 = (float)(0.25 * dt);
    __syncthreads();
    const int64_t lo = s_lo, hi = s_hi, gate = s_gate;
    // this thread's part of the population window [lo, hi], as chunk indices
    const int win_a = (int)max((int64_t)0, lo - s0), win_b = (int)min((int64_t)M - 1, hi - s0);
    const double* f = P.fields + I.field_off;
    double* out = P.outputs + I.out_off;
    double *o_t = out, *o_e = out + (S + 1), *o_src = out + 2 * (S + 1), *o_ptot = out + 3 * (S + 1),
           *o_pint = out + 4 * (S + 1), *o_x = out + 5 * (S + 1);
    {
        double v[1] = {0.0};
        for (int64_t j = t; j < n; j += T)
            if (j >= lo && j <= hi) v[0] += G.psi0[2 * j] * G.psi0[2 * j] + G.psi0[2 * j + 1] * G.psi0[2 * j + 1];
        block_sum<1, NW>(v, reinterpret_cast<double*>(red_hi));
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
    const float c_hi2 = 2.f * c_hi, c_lo2 = 2.f * c_lo, c12 = 2.f * c1;  // as in propagate_c64_kernel
    auto off_diag = [&](float v, float ir, float ii) -> cf {
        const float t1 = fmaf(c12, v, c_lo2);
        return cf{fmaf(-t1, ii, fmaf(-c_hi2, ii, ir)), fmaf(t1, ir, fmaf(c_hi2, ir, ii))};
    };
    // observables of output index ko (the state after step ko - 1), warp 0: two-sum of the
    // warps' partial sums into float pairs, kept in ring slot (ko - 1) mod KB
    auto obs_reduce = [&](int64_t ko) {
        const int c = lane >> 3, q = lane & 7;
        float hs = red_hi[q * 4 + c], ls = red_lo[q * 4 + c];
        for (int qq = q + 8; qq < NW; qq += 8) {  // warps beyond 8: fold into lanes 0..31 first
            float s2, e2;
            two_sum(hs, red_hi[qq * 4 + c], s2, e2);
            hs = s2;
            ls += red_lo[qq * 4 + c] + e2;
        }
#pragma unroll
        for (int d = 4; d >= 1; d >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hs, d);
            const float ol = __shfl_xor_sync(0xffffffffu, ls, d);
            float s2, e2;
            two_sum(hs, oh, s2, e2);
            hs = s2;
            ls += ol + e2;
        }
        const int j = (int)((ko - 1) % KB);
        if (q == 0) {
            obs_h[j][c] = hs;
            obs_l[j][c] = ls;
        }
        if (lane == 24) {
            float pi_sum = 0.f;
            for (int qq = 0; qq < NW; qq++) pi_sum += red_pi[qq];
            obs_pi[j] = pi_sum;
        }
    };
    // FP64 outputs of the cnt indices ending at k_last, one per lane: sourceterm -<V'> + F of
    // the step before, <x>, |<psi0|psi>|^2 and the window population (prop.c:266-300)
    auto obs_flush = [&](int64_t k_last, int cnt) {
        __syncwarp();
        if (lane < cnt) {
            const int64_t ko = k_last - cnt + 1 + lane, kp = ko - 1;
            const int j = (int)(kp % KB);
            double v[4];
#pragma unroll
            for (int c = 0; c < 4; c++) v[c] = (double)obs_h[j][c] + (double)obs_l[j][c];
            o_src[ko] = -v[0] + ((kp <= gate || kp >= I.n_field) ? 0.0 : __ldg(f + kp));
            o_x[ko] = v[1];
            o_ptot[ko] = fma(v[2], v[2], v[3] * v[3]);
            o_pint[ko] = (double)obs_pi[j];
        }
        __syncwarp();
    };
    cf yl[M], fg[M];

    for (int64_t k = 0; k < S; k++) {
        if (w == 0 && k > 0) {  // observables of the previous step
            obs_reduce(k);
            if ((k - 1) % KB == KB - 1) obs_flush(k, KB);
        }
        if (w == 1 && lane == 0) {
            tt += dt;
            o_t[k + 1] = tt;
            o_e[k + 1] = (k <= gate || k >= I.n_field) ? 0.0 : __ldg(f + k);
        }
        if (k % KB == 0) {
            // per-site phase factors of step k + w, each from its own angle: a recurrence in i
            // would carry the FP32 rounding of |e^{i F dt dx}| (1 +- 6e-8) as a bias growing
            // with i, and it would compound over the steps into a drift of the norm along each
            // chunk.  Read in pass 3, after the scans' barriers; refilled after the end-of-step
            // barrier of the block's last step.
            const int64_t ks = k + w;
            const double Fs = (ks <= gate || ks >= I.n_field || ks >= S) ? 0.0 : __ldg(f + ks);
            if (lane < M) {
                float sn, cs;
                sincosf((float)(Fs * dt * G.dx) * (float)lane, &sn, &cs);
                s_wtab[w][lane] = cf{cs, sn};
            }
            if (lane == 0) {
                const double fdt = Fs * dt;
                const float a_hi = (float)fdt;
                s_ahi[w] = a_hi;
                s_alo[w] = (float)(fdt - (double)a_hi);
            }
        }
        // ---- pass 1: right-hand side 2 M2 psi, local forward sweep, forward products F
        cf pm = (t == 0) ? cf{0.f, 0.f} : psi[(M - 1) * T + t - 1];
        cf pc = psi[t];
        float vl = (t == 0) ? 0.f : tab4[(M - 1) * T + t - 1].z;  // V of the site to the left
        cf yprev{0.f, 0.f}, Fp{1.f, 0.f};
#pragma unroll
        for (int i = 0; i < M; i++) {
            const int q = i * T + t;
            const cf pn = (i + 1 < M) ? psi[q + T] : ((t + 1 < T) ? psi[t + 1] : cf{0.f, 0.f});
            const cf r{fmaf(10.f, pc.re, pm.re + pn.re), fmaf(10.f, pc.im, pm.im + pn.im)};
            const float4 tb = tab4[q];
            const cf ib{tb.x, tb.y};
            const cf h = off_diag(vl, ib.re, ib.im);
            yprev = cfms(h, yprev, cmul(ib, r));
            yl[i] = yprev;
            Fp = cmul(Fp, cf{-h.re, -h.im});
            fg[i] = Fp;
            vl = tb.z;
            pm = pc;
            pc = pn;
        }
        const cf yin = scan_fwd<NW>(fg[M - 1], yprev, sc, sb);
        // ---- pass 2: forward correction, local backward sweep, backward products G
        cf unext{0.f, 0.f}, Gp{1.f, 0.f};
        float vr = (t == T - 1) ? 0.f : tab4[t + 1].z;  // V of the site to the right
#pragma unroll
        for (int i = M - 1; i >= 0; i--) {
            const int q = i * T + t;
            const cf y = cfma(fg[i], yin, yl[i]);
            const float4 tb = tab4[q];
            const cf g = off_diag(vr, tb.x, tb.y);
            unext = cfms(g, unext, y);
            yl[i] = unext;
            Gp = cmul(Gp, cf{-g.re, -g.im});
            fg[i] = Gp;
            vr = tb.z;
        }
        const cf uin = scan_bwd<NW>(fg[0], unext, sc + NW, sb + NW);
        // ---- pass 3: backward correction, CN update, phase, observables
        const int kb = (int)(k % KB);
        const float a_hi = s_ahi[kb], a_lo = s_alo[kb];
        const float th_hi = a_hi * xs_hi;
        const float th_lo = fmaf(a_hi, xs_hi, -th_hi) + fmaf(a_hi, xs_lo, a_lo * xs_hi);
        const float kk = rintf(th_hi * (float)kInvTwoPi);
        float red = fmaf(-kk, 6.28125f, th_hi);
        red = fmaf(-kk, 1.93500518798828125e-3f, red);
        red = fmaf(-kk, 3.0199159819370158e-07f, red) + th_lo;
        float sn, cs;
        sincosf(red, &sn, &cs);
        const cf phs{cs, sn};
        float ahi[4] = {0.f, 0.f, 0.f, 0.f}, alo[4] = {0.f, 0.f, 0.f, 0.f}, part[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < M; i++) {
            const int q = i * T + t;
            const cf u = cfma(fg[i], uin, yl[i]);  // u / 2
            const cf p0 = psi[q];
            const cf d{fmaf(2.f, u.re, -p0.re), fmaf(2.f, u.im, -p0.im)};
            const cf pn = cmul(cmul(phs, s_wtab[kb][i]), d);
            psi[q] = pn;
            const float n2 = fmaf(pn.re, pn.re, pn.im * pn.im);
            const float xj = fmaf(dxf, (float)i, xs_hi);
            const float4 tb = tab4[q];
            const float vj = tb.z, pj = tb.w;
            part[0] = fmaf(n2, -xj * vj * vj * vj, part[0]);  // -V' = -x V^3
            part[1] = fmaf(n2, xj, part[1]);
            part[2] = fmaf(pn.re, pj, part[2]);
            part[3] = fmaf(-pn.im, pj, part[3]);
            if ((i & 15) == 15 || i == M - 1) {
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    float s2, e2;
                    two_sum(ahi[c], part[c], s2, e2);
                    ahi[c] = s2;
                    alo[c] += e2;
                    part[c] = 0.f;
                }
            }
        }
        float pint = 0.f;
        for (int i = win_a; i <= win_b; i++) {  // the few sites of the window (own chunk)
            const cf p = psi[i * T + t];
            pint = fmaf(p.re, p.re, fmaf(p.im, p.im, pint));
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float oh = __shfl_xor_sync(0xffffffffu, ahi[c], d);
                const float ol = __shfl_xor_sync(0xffffffffu, alo[c], d);
                float s2, e2;
                two_sum(ahi[c], oh, s2, e2);
                ahi[c] = s2;
                alo[c] += ol + e2;
            }
            pint += __shfl_xor_sync(0xffffffffu, pint, d);
        }
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                red_hi[w * 4 + c] = ahi[c];
                red_lo[w * 4 + c] = alo[c];
            }
            red_pi[w] = pint;
        }
        if (I.snap_off >= 0 && P.snapshots) {  // prop.c:248-263
            int64_t slot = -1;
            if (k % I.snap_every == 0 && k / I.snap_every < I.n_snap - 1) slot = k / I.snap_every;
            if (k == S - 1) slot = I.n_snap - 1;
            if (slot >= 0) {
                double* sp = P.snapshots + I.snap_off + slot * 2 * n;
                for (int i = 0; i < M; i++)
                    if (s0 + i < n) {
                        sp[2 * (s0 + i)] = psi[i * T + t].re;
                        sp[2 * (s0 + i) + 1] = psi[i * T + t].im;
                    }
            }
        }
        __syncthreads();
    }
    if (w == 0 && S > 0) {  // observables of the last step, then the steps not yet converted
        obs_reduce(S);
        obs_flush(S, (int)((S - 1) % KB) + 1);
    }
    if (P.psi_final && I.psi_off >= 0) {
        double* pf = P.psi_final + I.psi_off;
        for (int i = 0; i < M; i++)
            if (s0 + i < n) {
                pf[2 * (s0 + i)] = psi[i * T + t].re;
                pf[2 * (s0 + i) + 1] = psi[i * T + t].im;
            }
    }
    __syncthreads();
}

template <int M, int T>  // 256 threads with M <= 16 fit twice on an SM (128 registers, <= 96 KB)
__global__ void __launch_bounds__(T, (T == 256 && M <= 16) ? 2 : 1) propagate_c64_smem_kernel(Args P)
{
    __shared__ int64_t s_inst;  // L sites x (1/beta re, im, V, psi0), then psi [L] complex float, dynamic
    const int t = threadIdx.x;
    if (t == 0) c64_s_grid = -1;
    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        if (G.m32 != M || (G.c64_threads ? G.c64_threads : kThreads) != T) {  // tables laid out for another shape
            nan_outputs(P, I, T);
            continue;
        }
        c64_smem_instance<M, T>(P, I, G);
    }
}

// The per-width bodies as separate (not inlined) functions for the width-dispatching kernel, so
// that each width keeps its own register allocation instead of the union of all six.  The
// records arrive by reference to the caller's stack; copies taken at entry keep their fields in
// registers inside the step loop instead of reloading them from local memory.
template <int M>
__device__ __noinline__ void c64_smem_instance_ni(const Args& P_, const mma_tdse_instance& I_,
                                                  const mma_tdse_grid& G_)
{
    const Args P = P_;
    const mma_tdse_instance I = I_;
    const mma_tdse_grid G = G_;
    c64_smem_instance<M, kThreads>(P, I, G);
}
template <int M>
__device__ __noinline__ void c64_reg_instance_ni(const Args& P_, const mma_tdse_instance& I_, const mma_tdse_grid& G_)
{
    const Args P = P_;
    const mma_tdse_instance I = I_;
    const mma_tdse_grid G = G_;
    c64_reg_instance<M>(P, I, G);
}

// Uneven batches in one launch: instances of every 256-thread table width (8 to 48 sites per
// thread) from one work queue, longest first.  Each CTA dispatches on its instance's width to
// the shared-memory form (M <= 32) or the register-resident form (M = 40, 48); the dynamic
// shared memory is the largest either needs (24 bytes per site at M = 32, 16 at M = 48), so
// one CTA runs per SM.  A CTA that changes width reloads the tables (s_grid is common to all).
__global__ void __launch_bounds__(kThreads, 1) propagate_c64_mixed_kernel(Args P)
{
    __shared__ int64_t s_inst;
    const int t = threadIdx.x;
    if (t == 0) c64_s_grid = -1;
    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        if ((G.c64_threads ? G.c64_threads : kThreads) != kThreads) {
            nan_outputs(P, I, kThreads);
            continue;
        }
        switch (G.m32) {
        case 8: c64_smem_instance_ni<8>(P, I, G); break;
        case 16: c64_smem_instance_ni<16>(P, I, G); break;
        case 24: c64_smem_instance_ni<24>(P, I, G); break;
        case 32: c64_smem_instance_ni<32>(P, I, G); break;
        case 40: c64_reg_instance_ni<40>(P, I, G); break;
        case 48: c64_reg_instance_ni<48>(P, I, G); break;
        default: nan_outputs(P, I, kThreads); break;
        }
    }
}

// Complex64 tables from the FP64 grid data, laid out for T = c64_threads threads x M32 sites.
__global__ void __launch_bounds__(kThreads) build_c64_kernel(const mma_tdse_grid* grids)
{
    const mma_tdse_grid G = grids[blockIdx.x];
    const int64_t T = G.c64_threads ? G.c64_threads : kThreads;
    const int64_t n = G.n, m = G.m, Lm = m * kThreads, M = G.m32, L = M * T;
    const cd* ctab = reinterpret_cast<const cd*>(G.cn_tab);
    for (int64_t q = threadIdx.x; q < L; q += blockDim.x) {
        const int64_t i = q / T, t = q % T, j = t * M + i;
        float v[T_SLOTS] = {0.f, 0.f, 0.f, 0.f};
        if (j < n) {
            const int64_t q64 = (j % m) * kThreads + j / m;  // FP64 table layout
            const cd ib6 = ctab[0 * Lm + q64];
            const double vj = -1.0 / sqrt(G.trg_a * G.trg_a + G.x[j] * G.x[j]);
            v[T_IBRE] = (float)(0.5 * ib6.re);  // half of 1/beta: exact scaling of the rounded value
            v[T_IBIM] = (float)(0.5 * ib6.im);
            v[T_V] = (float)vj;
            v[T_PSI0] = (float)G.psi0[2 * j];
        }
#pragma unroll
        for (int s = 0; s < T_SLOTS; s++) G.c64_tab[s * L + q] = v[s];
    }
}

}  // namespace c64
}  // namespace mma

using namespace mma;

// Shapes (CTA threads T, sites per thread M) the complex64 form has kernels for.
static bool c64_shape_ok(int64_t T, int64_t M)
{
    if (T == kThreads) return M == 8 || M == 16 || M == 24 || M == 32 || M == 40 || M == 48;
    if (T == 512) return M == 8 || M == 16;
    if (T == 1024) return M == 8;
    return false;
}

extern "C" int mma_tdse_c64_shape_ok(int cta_threads, int m32)
{
    return c64_shape_ok(cta_threads ? cta_threads : kThreads, m32) ? 1 : 0;
}

extern "C" int mma_tdse_build_c64_tables(const mma_tdse_grid* grids_dev, const mma_tdse_grid* grids_host, int n_grids,
                                         void* stream)
{
    if (n_grids <= 0 || !grids_dev || !grids_host) return MMA_ERR_ARG;
    for (int g = 0; g < n_grids; g++) {
        const mma_tdse_grid& G = grids_host[g];
        const int64_t T = G.c64_threads ? G.c64_threads : kThreads;
        if (!G.c64_tab || !c64_shape_ok(T, G.m32) || G.m32 * T < G.n) return MMA_ERR_ARG;
    }
    c64::build_c64_kernel<<<n_grids, kThreads, 0, (cudaStream_t)stream>>>(grids_dev);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

namespace {
template <int M, int T>
int launch_c64(const c64::Args& A, int ctas, cudaStream_t st)
{
    if constexpr (M <= 32) {  // wavefunction in shared memory next to the tables
        const size_t smem = (size_t)c64::T_SLOTS * T * M * sizeof(float) + (size_t)T * M * 8;
        cudaFuncSetAttribute(c64::propagate_c64_smem_kernel<M, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        c64::propagate_c64_smem_kernel<M, T><<<ctas, T, smem, st>>>(A);
    } else {  // wavefunction in registers, five-pass re-sweep (T = 256)
        const size_t smem = (size_t)c64::T_SLOTS * kThreads * M * sizeof(float);
        cudaFuncSetAttribute(c64::propagate_c64_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        c64::propagate_c64_kernel<M><<<ctas, kThreads, smem, st>>>(A);
    }
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
}  // namespace

// Dynamic shared memory of the width-dispatching kernel: the larger of the shared-memory form at
// M = 32 (tables and psi, 24 bytes per site) and the register-resident form at M = 48 (tables,
// 16 bytes per site).
static size_t mixed_smem_bytes()
{
    const size_t a = (size_t)c64::T_SLOTS * kThreads * 32 * sizeof(float) + (size_t)kThreads * 32 * 8;
    const size_t b = (size_t)c64::T_SLOTS * kThreads * 48 * sizeof(float);
    return a > b ? a : b;
}

// CTAs of the complex64 form resident at once for tables laid out for (cta_threads, m32): the
// occupancy of that kernel shape (two per SM for 256 threads with m32 <= 16: 96 KB of shared
// memory and 128 registers per thread; one otherwise) times the SMs.
extern "C" int mma_tdse_c64_default_ctas(int m32, int cta_threads)
{
    const int T = cta_threads ? cta_threads : kThreads;
    int dev = 0, sms = 0, per_sm = 1;
    if (m32 == 0 && T == kThreads) {  // the width-dispatching kernel: one CTA per SM
        if (cudaGetDevice(&dev) != cudaSuccess) return 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return sms;
    }
    if (!c64_shape_ok(T, m32) || cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (T == kThreads && m32 <= 16) {
        const size_t smem = (size_t)c64::T_SLOTS * T * m32 * sizeof(float) + (size_t)T * m32 * 8;
        const void* fn = m32 == 8 ? (const void*)c64::propagate_c64_smem_kernel<8, kThreads>
                                  : (const void*)c64::propagate_c64_smem_kernel<16, kThreads>;
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    }
    return sms * per_sm;
}

// Launch of the complex64 form (called by mma_tdse_propagate_ex for precision 1): every
// instance's grid must have tables of shape (cta_threads, m32).
extern "C" int mma_tdse_propagate_c64_impl(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                           const mma_tdse_buffers* bufs, int m32, int cta_threads, int grid_ctas,
                                           void* stream)
{
    c64::Args A{insts, n_inst, grids, bufs->fields, bufs->outputs, bufs->psi_final, bufs->snapshots, bufs->counter};
    cudaStream_t st = (cudaStream_t)stream;
    const int T = cta_threads ? cta_threads : kThreads;
    if (m32 == 0) {  // every 256-thread table width in one launch
        if (T != kThreads) return MMA_ERR_UNSUPPORTED;
        if (cudaMemsetAsync(bufs->counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
        const size_t smem = mixed_smem_bytes();
        cudaFuncSetAttribute(c64::propagate_c64_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        c64::propagate_c64_mixed_kernel<<<grid_ctas, kThreads, smem, st>>>(A);
        return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
    }
    if (!c64_shape_ok(T, m32)) return MMA_ERR_TOO_LARGE;
    if (cudaMemsetAsync(bufs->counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    if (T == 512) return m32 == 8 ? launch_c64<8, 512>(A, grid_ctas, st) : launch_c64<16, 512>(A, grid_ctas, st);
    if (T == 1024) return launch_c64<8, 1024>(A, grid_ctas, st);
    switch (m32) {
        case 8: return launch_c64<8, kThreads>(A, grid_ctas, st);
        case 16: return launch_c64<16, kThreads>(A, grid_ctas, st);
        case 24: return launch_c64<24, kThreads>(A, grid_ctas, st);
        case 32: return launch_c64<32, kThreads>(A, grid_ctas, st);
        case 40: return launch_c64<40, kThreads>(A, grid_ctas, st);
        case 48: return launch_c64<48, kThreads>(A, grid_ctas, st);
        default: return MMA_ERR_TOO_LARGE;
    }
}
