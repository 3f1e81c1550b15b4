// tdse_df64.cu -- float-float ("df64") form of the TDSE propagation: the FP64 Crank-Nicolson-
// Numerov step (prop.c:115-347, the same tables and partitioned solve as propagate_fp64_kernel)
// carried out in double-word FP32 arithmetic.
//
// On this GPU FP32 runs at about 62x the FP64 rate, so a double-word operation of 6-25 FP32
// instructions still outruns one FP64 operation.  A value is a pair (hi, lo) of floats with
// |lo| <= ulp(hi)/2, about 48 significant bits; every operation below is built from two
// error-free transformations:
//   * TwoSum (Knuth): s + e = a + b exactly, s = fl(a + b);
//   * TwoProduct with an FMA: p + e = a b exactly, p = fl(a b), e = fma(a, b, -p);
// with the accurate double-word addition of Joldes, Muller and Popescu ("Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic", ACM TOMS 2017, Alg. 6):
// relative error about 3 u^2 (u = 2^-24).  Products and sums of products fold their low-order
// terms with FMAs before one final renormalisation.
//
// Layout as in the FP64 kernel: site j = t m + i at q = i T + t; the tables are the FP64 tables
// split once per grid into (hi, lo) float pairs (mma_tdse_build_df_tables).  psi and the sweep
// buffer live in the caller's scratch (L2-resident, 16 bytes per site each) rather than in shared
// memory, so that two 256-thread CTAs fit on an SM: the double-word operations are long
// dependency chains and 16 warps hide them better than 8 (measured 27% faster on config 1).
// Each pass reads its operands through a small cp.async ring in shared memory, two sites ahead,
// which hides the L2 latency without registers (30% faster at one CTA per SM, 9% at two).
// No warp carries serial FP64 work into the scan barriers (a 32-lane FP64 instruction holds a
// sub-partition's FP64 unit for about 64 cycles): the phase factors come from one FP64 sincos
// per thread for 25 steps at a time, and the observables' warp sums stay double-word until
// lanes of warp 0 convert them.
#include <cuda_runtime.h>

#include "../../include/mma_tdse.h"
#include "common.cuh"
#include "tdse_step.cuh"

namespace mma {
namespace dfk {

struct df {
    float hi, lo;
};
struct cdf {
    df re, im;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)  // |a| >= |b|
{
    s = a + b;
    e = b - (s - a);
}
__device__ __forceinline__ df renorm(float s, float e)
{
    df r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
// x + y (Joldes, Muller, Popescu 2017, Algorithm 6)
__device__ __forceinline__ df add(df x, df y)
{
    float sh, sl, th, tl;
    two_sum(x.hi, y.hi, sh, sl);
    two_sum(x.lo, y.lo, th, tl);
    sl += th;
    fast_two_sum(sh, sl, sh, sl);
    sl += tl;
    return renorm(sh, sl);
}
__device__ __forceinline__ df neg(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df sub(df x, df y) { return add(x, neg(y)); }
// x y
__device__ __forceinline__ df mul(df x, df y)
{
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return renorm(p, e);
}
// a b + c d + z (products exact to first order, one accurate sum with z)
__device__ __forceinline__ df dot2_add(df a, df b, df c, df d, df z)
{
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    eq = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, eq));
    float s1, t1, s2, t2;
    two_sum(p, q, s1, t1);
    two_sum(s1, z.hi, s2, t2);
    const float e = ((t1 + t2) + (ep + eq)) + z.lo;
    return renorm(s2, e);
}
// Results consumed only as operands of the next double-word product or sum (never stored, never
// carried from site to site) skip the final renormalisation: their (hi, lo) come straight from
// the error-free transformations, |lo| at most a few ulp(hi), which the products below take
// exactly to first order like any pair.
// a b + c d, unnormalised
__device__ __forceinline__ df dot2_u(df a, df b, df c, df d)
{
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    eq = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, eq));
    float s1, t1;
    two_sum(p, q, s1, t1);
    return df{s1, t1 + (ep + eq)};
}
// a b + c d
__device__ __forceinline__ df dot2(df a, df b, df c, df d)
{
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    eq = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, eq));
    float s1, t1;
    two_sum(p, q, s1, t1);
    return renorm(s1, t1 + (ep + eq));
}
// a b + c d + z + w, one renormalisation (the four leading terms by three TwoSums, every
// low-order term folded once)
__device__ __forceinline__ df dot2_add2(df a, df b, df c, df d, df z, df w)
{
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    eq = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, eq));
    float s1, t1, s2, t2, s3, t3;
    two_sum(p, q, s1, t1);
    two_sum(z.hi, w.hi, s2, t2);
    two_sum(s1, s2, s3, t3);
    return df{s3, ((t1 + t2) + t3) + ((ep + eq) + (z.lo + w.lo))};  // unnormalised (feeds cmul)
}
// Accumulators of a site loop: hi takes each term's leading part by a TwoSum, lo gathers every
// low-order part; renormalised once after the loop (lo stays far below ulp(hi) over a chunk).
// acc += a b
__device__ __forceinline__ void acc_mul(df& acc, df a, df b)
{
    const float p = a.hi * b.hi;
    float ep = fmaf(a.hi, b.hi, -p);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.hi = s;
    acc.lo += e + ep;
}
// acc += a b + c d
__device__ __forceinline__ void acc_dot2(df& acc, df a, df b, df c, df d)
{
    const float p = a.hi * b.hi, q = c.hi * d.hi;
    float ep = fmaf(a.hi, b.hi, -p), eq = fmaf(c.hi, d.hi, -q);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    eq = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, eq));
    float s1, t1, s2, t2;
    two_sum(p, q, s1, t1);
    two_sum(acc.hi, s1, s2, t2);
    acc.hi = s2;
    acc.lo += (t1 + t2) + (ep + eq);
}
// a b + z
__device__ __forceinline__ df mul_add(df a, df b, df z)
{
    const float p = a.hi * b.hi;
    float ep = fmaf(a.hi, b.hi, -p);
    ep = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, ep));
    float s1, t1;
    two_sum(p, z.hi, s1, t1);
    return renorm(s1, (t1 + ep) + z.lo);
}
// 10 p + a + b (the Numerov right-hand side), one renormalisation
__device__ __forceinline__ df ten_sum(df p, df a, df b)
{
    const float x = 10.f * p.hi;
    const float ex = fmaf(10.f, p.lo, fmaf(10.f, p.hi, -x));
    float s1, t1, s2, t2;
    two_sum(a.hi, b.hi, s1, t1);
    two_sum(x, s1, s2, t2);
    return df{s2, ((t1 + t2) + ex) + (a.lo + b.lo)};  // unnormalised (feeds cmul)
}
__device__ __forceinline__ cdf cmul(cdf a, cdf b)
{
    return cdf{dot2(a.re, b.re, neg(a.im), b.im), dot2(a.re, b.im, a.im, b.re)};
}
__device__ __forceinline__ cdf cmul_u(cdf a, cdf b)  // unnormalised (feeds a sum)
{
    return cdf{dot2_u(a.re, b.re, neg(a.im), b.im), dot2_u(a.re, b.im, a.im, b.re)};
}
// z + a b
__device__ __forceinline__ cdf cfma(cdf a, cdf b, cdf z)
{
    return cdf{dot2_add(a.re, b.re, neg(a.im), b.im, z.re), dot2_add(a.re, b.im, a.im, b.re, z.im)};
}
// z - a b
__device__ __forceinline__ cdf cfms(cdf a, cdf b, cdf z)
{
    return cdf{dot2_add(neg(a.re), b.re, a.im, b.im, z.re), dot2_add(neg(a.re), b.im, neg(a.im), b.re, z.im)};
}
__device__ __forceinline__ cdf cadd(cdf a, cdf b) { return cdf{add(a.re, b.re), add(a.im, b.im)}; }
__device__ __forceinline__ cdf csub(cdf a, cdf b) { return cdf{sub(a.re, b.re), sub(a.im, b.im)}; }
__device__ __forceinline__ df from_d(double v)
{
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
}
__device__ __forceinline__ double to_d(df v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ cdf ld(const float4* p) { const float4 v = *p; return cdf{{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ void st(float4* p, cdf v) { *p = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo); }

// 16-byte global -> shared copy (L2 only), grouped per iteration; a thread reads back only what it
// copied itself, so completing its own groups (cp.async.wait_group) is the only wait
__device__ __forceinline__ void cp16(float4* dst_smem, const float4* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ df shfl_up_df(df v, int d)
{
    return df{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}
__device__ __forceinline__ df shfl_dn_df(df v, int d)
{
    return df{__shfl_down_sync(0xffffffffu, v.hi, d), __shfl_down_sync(0xffffffffu, v.lo, d)};
}
__device__ __forceinline__ df shfl_xor_df(df v, int d)
{
    return df{__shfl_xor_sync(0xffffffffu, v.hi, d), __shfl_xor_sync(0xffffffffu, v.lo, d)};
}
__device__ __forceinline__ cdf shup(cdf v, int d) { return cdf{shfl_up_df(v.re, d), shfl_up_df(v.im, d)}; }
__device__ __forceinline__ cdf shdn(cdf v, int d) { return cdf{shfl_dn_df(v.re, d), shfl_dn_df(v.im, d)}; }

// exclusive CTA scans of the affine maps Y_t = b_t + c_t Y_{t-1} (forward) and
// U_t = b_t + c_t U_{t+1} (backward), as scan_forward / scan_backward (tdse_solver.cuh)
__device__ cdf scan_fwd(cdf c, cdf b, cdf* sc, cdf* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const cdf cp = shup(c, d), bp = shup(b, d);
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
    cdf yw{{0.f, 0.f}, {0.f, 0.f}};
    for (int q = 0; q < w; q++) yw = cfma(sc[q], yw, sb[q]);
    const cdf cp = shup(c, 1), bp = shup(b, 1);
    return lane == 0 ? yw : cfma(cp, yw, bp);
}

__device__ cdf scan_bwd(cdf c, cdf b, cdf* sc, cdf* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const cdf cp = shdn(c, d), bp = shdn(b, d);
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
    cdf uw{{0.f, 0.f}, {0.f, 0.f}};
    for (int q = kWarps - 1; q > w; q--) uw = cfma(sc[q], uw, sb[q]);
    const cdf cp = shdn(c, 1), bp = shdn(b, 1);
    return lane == 31 ? uw : cfma(cp, uw, bp);
}

// The step's observables from the per-warp double-word partial sums (lane c < 5 sums column c
// over the warps), in FP64 from there: sourceterm -<V'> + F, <x>, |<psi0|psi>|^2 and the window
// population (prop.c:266-300, tools_algorithmic.c:19-43).  Called by one warp.
__device__ __forceinline__ void observables_out(const df* redf, int lane, int64_t k, double F_prev, double* o_src,
                                                double* o_x, double* o_ptot, double* o_pint)
{
    df s{0.f, 0.f};
    if (lane < 5)
#pragma unroll
        for (int q = 0; q < kWarps; q++) s = add(s, redf[q * 5 + lane]);
    const double v = to_d(s);
    const double v3 = __shfl_down_sync(0xffffffffu, v, 1);  // lane 2 gets the imaginary projection
    if (lane == 0) o_src[k] = -v + F_prev;
    if (lane == 1) o_x[k] = v;
    if (lane == 2) o_ptot[k] = v * v + v3 * v3;
    if (lane == 4) o_pint[k] = v;
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
    float4* scratch;  // per CTA: yl [L], then psi [L]
    int64_t max_L;
};

constexpr int kPow = 8;  // e^{i F dt M dx 2^b}, b < 8: the chunk-start phases of 256 threads
constexpr int kPhase = kPow + 2;  // phase factors per step
constexpr int kPhaseSteps = kThreads / kPhase;  // steps whose factors one pass of the CTA computes
// Operand ring: each pass copies the operands of site i + kDepth - 1 into shared memory while it
// computes site i (kSlots float4 per site at most, pass 3), so the L2 latency of psi, the sweep
// buffer and the tables is hidden without holding registers.
constexpr int kDepth = 3, kSlots = 5;
constexpr int kRingBytes = kDepth * kSlots * kThreads * 16;  // 61,440 bytes per CTA

__global__ void __launch_bounds__(kThreads, 2) propagate_df64_kernel(Args P)
{
    extern __shared__ float4 ring[];  // [kDepth][kSlots][kThreads]
    __shared__ cdf sc[2 * kWarps], sb[2 * kWarps];
    __shared__ double red[kWarps];
    __shared__ df redf[kWarps * 5];  // per warp: -<V'>, <x>, <psi0|psi> (re, im), window population
    // per step of the current block of kPhaseSteps: e^{i F dt x_0}, e^{i F dt dx}, e^{i F dt M dx 2^b}
    __shared__ cdf s_pow[kPhaseSteps][kPhase];
    __shared__ int64_t s_inst, s_gate, s_lo, s_hi;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    float4* yl = P.scratch + blockIdx.x * P.max_L;
    float4* psi = P.scratch + (gridDim.x + blockIdx.x) * P.max_L;

    for (;;) {
        if (t == 0) s_inst = atomicAdd(P.counter, 1);
        __syncthreads();
        const int64_t inst = s_inst;
        if (inst >= P.n_inst) break;
        const mma_tdse_instance I = P.insts[inst];
        const mma_tdse_grid G = P.grids[I.grid];
        const int64_t n = G.n, m = G.m, L = m * kThreads, S = I.n_steps;
        const float4* tab = reinterpret_cast<const float4*>(G.df_tab);
        const float4 *IB = tab + CN_IB6 * L, *HH = tab + CN_H * L, *FF = tab + CN_F * L, *GG_ = tab + CN_G * L,
                     *GP = tab + CN_GG * L, *P0 = tab + CN_PSI0 * L, *GVX = tab + CN_GVX * L;
        const double* f = P.fields + I.field_off;
        double* out = P.outputs + I.out_off;
        double *o_t = out, *o_e = out + (S + 1), *o_src = out + 2 * (S + 1), *o_ptot = out + 3 * (S + 1),
               *o_pint = out + 4 * (S + 1), *o_x = out + 5 * (S + 1);
        const double dt = G.dt, dx = G.dx;
        if (t == 0) {
            s_gate = gate_index(f, I.n_field, S, I.gate_floor);
            const int64_t num_r = n - 1;  // PopInt window (tools_algorithmic.c:19-43)
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
        for (int64_t i = 0; i < m; i++) psi[i * kThreads + t] = P0[i * kThreads + t];
        __syncthreads();
        const int64_t lo = s_lo, hi = s_hi, gate = s_gate;
        const int64_t s0 = t * m;
        {   // initial window population (prop.c:87-93), FP64 from the FP64 ground state
            double v[1] = {0.0};
            for (int64_t j = t; j < n; j += kThreads)
                if (j >= lo && j <= hi) v[0] += G.psi0[2 * j] * G.psi0[2 * j] + G.psi0[2 * j + 1] * G.psi0[2 * j + 1];
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
        double tt = I.tmin, Fprev = 0.0;
        const double x0 = G.x[0];
        for (int64_t k = 0; k < S; k++) {
            const double Fk = (k <= gate || k >= I.n_field) ? 0.0 : f[k];
            if (w == 0) {
                if (k > 0) observables_out(redf, lane, k, Fprev, o_src, o_x, o_ptot, o_pint);
                if (lane == 0) {
                    tt += dt;
                    o_t[k + 1] = tt;
                    o_e[k + 1] = Fk;
                }
            }
            Fprev = Fk;
            // the phase factors of the next kPhaseSteps steps in FP64, one angle per thread, so
            // that the FP64 pipe's work is spread evenly over the warps: e^{i F dt x_0},
            // e^{i F dt dx} and e^{i F dt m dx 2^b}
            if (k % kPhaseSteps == 0 && t < kPhaseSteps * kPhase) {
                const int a = t % kPhase;
                const int64_t ks = k + t / kPhase;
                const double Fs = (ks <= gate || ks >= I.n_field || ks >= S) ? 0.0 : f[ks];
                const double ang = a == 0 ? Fs * dt * x0 : (a == 1 ? Fs * dt * dx
                                                                   : Fs * dt * (double)m * dx * (double)(1 << (a - 2)));
                double sn, cs;
                sincos(ang, &sn, &cs);
                s_pow[t / kPhase][a] = cdf{from_d(cs), from_d(sn)};
            }
            // ---- pass 1: local forward sweep of the right-hand side 2 M2 psi
            const cdf zero{{0.f, 0.f}, {0.f, 0.f}};
            const int mi = (int)m;  // sites per thread: 32-bit indices in the site loops
            float4* const my = ring + t;
            constexpr int kStage = kSlots * kThreads;
            // site i's operands: psi of site i + 1 (the next thread's first site after the last),
            // H and 1/(2 beta)
            auto issue1 = [&](int i, float4* r) {
                const int q = i * kThreads + t;
                cp16(r, (i + 1 < mi) ? psi + q + kThreads : psi + (t + 1 < kThreads ? t + 1 : t));
                cp16(r + kThreads, HH + q);
                cp16(r + 2 * kThreads, IB + q);
            };
#pragma unroll
            for (int d = 0; d < kDepth - 1; d++) {
                if (d < mi) issue1(d, my + d * kStage);
                cp_commit();
            }
            cdf pm = (t == 0) ? zero : ld(psi + (m - 1) * kThreads + t - 1);
            cdf pc = ld(psi + t);
            cdf yprev = zero;
            int su = 0;  // ring stage of the current site; the stage before it is refilled
            for (int i = 0; i < mi; i++) {
                float4* const r = my + su * kStage;
                if (i + kDepth - 1 < mi) issue1(i + kDepth - 1, my + (su == 0 ? kDepth - 1 : su - 1) * kStage);
                cp_commit();
                cp_wait<kDepth - 1>();
                const cdf pn = (i + 1 < mi || t + 1 < kThreads) ? ld(r) : zero;
                const cdf r2{ten_sum(pc.re, pm.re, pn.re), ten_sum(pc.im, pm.im, pn.im)};
                yprev = cfms(ld(r + kThreads), yprev, cmul_u(ld(r + 2 * kThreads), r2));
                st(yl + i * kThreads + t, yprev);
                pm = pc;
                pc = pn;
                su = su + 1 == kDepth ? 0 : su + 1;
            }
            const cdf yin = scan_fwd(ld(FF + (m - 1) * kThreads + t), yprev, sc, sb);
            // ---- pass 2: forward correction, local backward sweep
            auto issue2 = [&](int i, float4* r) {  // F, y and G of site i
                const int q = i * kThreads + t;
                cp16(r, FF + q);
                cp16(r + kThreads, yl + q);
                cp16(r + 2 * kThreads, GG_ + q);
            };
#pragma unroll
            for (int d = 0; d < kDepth - 1; d++) {
                if (d < mi) issue2(mi - 1 - d, my + d * kStage);
                cp_commit();
            }
            cdf unext = zero;
            su = 0;
            for (int j = 0; j < mi; j++) {  // site i = mi - 1 - j
                float4* const r = my + su * kStage;
                if (j + kDepth - 1 < mi) issue2(mi - kDepth - j, my + (su == 0 ? kDepth - 1 : su - 1) * kStage);
                cp_commit();
                cp_wait<kDepth - 1>();
                const cdf y = cfma(ld(r), yin, ld(r + kThreads));
                unext = cfms(ld(r + 2 * kThreads), unext, y);
                st(yl + (mi - 1 - j) * kThreads + t, unext);
                su = su + 1 == kDepth ? 0 : su + 1;
            }
            const cdf uin = scan_bwd(ld(GP + t), unext, sc + kWarps, sb + kWarps);
            // ---- pass 3: backward correction, CN update, phase e^{+i F dt x}, observables
            const cdf* pw = s_pow[k % kPhaseSteps];
            cdf ph = pw[0];  // e^{i F dt x_0} (e^{i F dt m dx})^t = e^{i F dt x_{s0}}
#pragma unroll
            for (int b = 0; b < kPow; b++)
                if (t & (1 << b)) ph = cmul(ph, pw[2 + b]);
            const cdf z = pw[1];
            df acc[5] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            auto issue3 = [&](int i, float4* r) {  // G, u, psi, (-V', x) and psi0 of site i
                const int q = i * kThreads + t;
                cp16(r, GP + q);
                cp16(r + kThreads, yl + q);
                cp16(r + 2 * kThreads, psi + q);
                cp16(r + 3 * kThreads, GVX + q);
                cp16(r + 4 * kThreads, P0 + q);
            };
#pragma unroll
            for (int d = 0; d < kDepth - 1; d++) {
                if (d < mi) issue3(d, my + d * kStage);
                cp_commit();
            }
            su = 0;
            for (int i = 0; i < mi; i++) {
                float4* const r = my + su * kStage;
                if (i + kDepth - 1 < mi) issue3(i + kDepth - 1, my + (su == 0 ? kDepth - 1 : su - 1) * kStage);
                cp_commit();
                cp_wait<kDepth - 1>();
                su = su + 1 == kDepth ? 0 : su + 1;
                const int q = i * kThreads + t;
                const cdf gp = ld(r), yv = ld(r + kThreads), po = ld(r + 2 * kThreads);
                // u - psi with u = G u_in + y, the CN update before the phase
                const cdf d{dot2_add2(gp.re, uin.re, neg(gp.im), uin.im, yv.re, neg(po.re)),
                            dot2_add2(gp.re, uin.im, gp.im, uin.re, yv.im, neg(po.im))};
                const cdf pn = cmul(ph, d);
                st(psi + q, pn);
                ph = cmul(ph, z);
                const df n2 = dot2_u(pn.re, pn.re, pn.im, pn.im);
                const cdf gx = ld(r + 3 * kThreads), p0 = ld(r + 4 * kThreads);
                acc_mul(acc[0], n2, gx.re);
                acc_mul(acc[1], n2, gx.im);
                acc_dot2(acc[2], pn.re, p0.re, pn.im, p0.im);
                acc_dot2(acc[3], pn.re, p0.im, neg(pn.im), p0.re);
            }
#pragma unroll
            for (int c = 0; c < 4; c++) acc[c] = renorm(acc[c].hi, acc[c].lo);
            acc[4] = df{0.f, 0.f};  // the few sites of the population window in this chunk
            for (int64_t j = (lo > s0 ? lo : s0); j <= hi && j < s0 + m; j++) {
                const cdf v = ld(psi + (j - s0) * kThreads + t);
                acc[4] = add(acc[4], dot2(v.re, v.re, v.im, v.im));
            }
            // warp sums in double-word arithmetic; across warps at the next step (observables_out)
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1)
#pragma unroll
                for (int c = 0; c < 5; c++) acc[c] = add(acc[c], shfl_xor_df(acc[c], d));
            if (lane == 0)
#pragma unroll
                for (int c = 0; c < 5; c++) redf[w * 5 + c] = acc[c];
            if (I.snap_off >= 0 && P.snapshots) {  // prop.c:248-263
                int64_t slot = -1;
                if (k % I.snap_every == 0 && k / I.snap_every < I.n_snap - 1) slot = k / I.snap_every;
                if (k == S - 1) slot = I.n_snap - 1;
                if (slot >= 0) {
                    double* sp = P.snapshots + I.snap_off + slot * 2 * n;
                    for (int64_t i = 0; i < m; i++)
                        if (s0 + i < n) {
                            const cdf v = ld(psi + i * kThreads + t);
                            sp[2 * (s0 + i)] = to_d(v.re);
                            sp[2 * (s0 + i) + 1] = to_d(v.im);
                        }
                }
            }
            __syncthreads();
        }
        if (w == 0) observables_out(redf, lane, S, Fprev, o_src, o_x, o_ptot, o_pint);
        if (P.psi_final && I.psi_off >= 0) {
            double* pf = P.psi_final + I.psi_off;
            for (int64_t i = 0; i < m; i++)
                if (s0 + i < n) {
                    const cdf v = ld(psi + i * kThreads + t);
                    pf[2 * (s0 + i)] = to_d(v.re);
                    pf[2 * (s0 + i) + 1] = to_d(v.im);
                }
        }
        __syncthreads();
    }
}

// the FP64 CN tables of a grid split into (hi, lo) float pairs, slot by slot in the same layout
__global__ void __launch_bounds__(kThreads) build_df_kernel(const mma_tdse_grid* grids)
{
    const mma_tdse_grid G = grids[blockIdx.x];
    const int64_t L = G.m * kThreads, cnt = (int64_t)CN_SLOTS * L;  // complex entries
    const cd* src = reinterpret_cast<const cd*>(G.cn_tab);
    float4* dst = reinterpret_cast<float4*>(G.df_tab);
    for (int64_t q = threadIdx.x; q < cnt; q += blockDim.x) {
        const cd v = src[q];
        const df re = from_d(v.re), im = from_d(v.im);
        dst[q] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
}

}  // namespace dfk
}  // namespace mma

using namespace mma;

extern "C" int mma_tdse_build_df_tables(const mma_tdse_grid* grids_dev, const mma_tdse_grid* grids_host, int n_grids,
                                        void* stream)
{
    if (n_grids <= 0 || !grids_dev || !grids_host) return MMA_ERR_ARG;
    for (int g = 0; g < n_grids; g++)
        if (!grids_host[g].df_tab || !grids_host[g].cn_tab) return MMA_ERR_ARG;
    dfk::build_df_kernel<<<n_grids, kThreads, 0, (cudaStream_t)stream>>>(grids_dev);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

// CTAs of the float-float form resident at once (two per SM), and the scratch they need:
// per CTA the sweep buffer and psi, 16 bytes per site each.
static bool df64_smem_attr()
{
    return cudaFuncSetAttribute(dfk::propagate_df64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                dfk::kRingBytes) == cudaSuccess;
}

extern "C" int mma_tdse_df64_default_ctas()
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || !df64_smem_attr()) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dfk::propagate_df64_kernel, kThreads, dfk::kRingBytes);
    return sms * (per_sm > 0 ? per_sm : 1);
}

extern "C" size_t mma_tdse_df64_scratch_bytes(int max_m, int grid_ctas)
{
    return (size_t)max_m * kThreads * 16 * 2 * (size_t)grid_ctas;
}

// Launch of the float-float form (called by mma_tdse_propagate_ex for precision 2).
extern "C" int mma_tdse_propagate_df64_impl(const mma_tdse_instance* insts, int n_inst, const mma_tdse_grid* grids,
                                            const mma_tdse_buffers* bufs, int max_m, int grid_ctas, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(bufs->counter, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    dfk::Args A{insts, n_inst, grids, bufs->fields, bufs->outputs, bufs->psi_final, bufs->snapshots, bufs->counter,
                reinterpret_cast<float4*>(bufs->scratch), (int64_t)max_m * kThreads};
    if (!df64_smem_attr()) return MMA_ERR_CUDA;
    dfk::propagate_df64_kernel<<<grid_ctas, kThreads, dfk::kRingBytes, st>>>(A);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
