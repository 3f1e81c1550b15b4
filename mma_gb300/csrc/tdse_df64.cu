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
// The complex values of the site loops run as packed FP32x2 pairs, (re.hi, im.hi) and (re.lo,
// im.lo): real and imaginary parts take the same operations, so one FP32x2 instruction does two.
// Against the same arithmetic written per component: 27% fewer instructions, the same bits,
// 2.5% faster (the kernel is then bound by the latency of the sweeps' dependency chains).
//
// Layout as in the FP64 kernel: site j = t m + i at q = i T + t; the tables are the FP64 tables
// split once per grid into float4 (re.hi, im.hi, re.lo, im.lo) (mma_tdse_build_df_tables).  psi
// and the sweep buffer live in the caller's scratch (L2-resident, 16 bytes per site each) rather than in shared
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
__device__ __forceinline__ df from_d(double v)
{
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
}
__device__ __forceinline__ double to_d(df v) { return (double)v.hi + (double)v.lo; }

// ------------------------------------------------------------------ packed complex double-words
// A complex double-word value as two FP32x2 pairs: h = (re.hi, im.hi), l = (re.lo, im.lo), stored
// as the float4 (re.hi, im.hi, re.lo, im.lo).  Real and imaginary parts go through the same
// sequence of operations, so one packed FP32x2 instruction does the work of two FP32 ones; each
// lane gets exactly the IEEE operations of the component-wise double-word formula stated beside
// the routine, in the same order.  A complex product a b takes a's parts as broadcast pairs and
// b as (b) and i b = (-b.im, b.re), so lane re gets a.re b.re + a.im (-b.im) and lane im
// a.re b.im + a.im b.re.
struct pk {
    float2 h, l;
};
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(*reinterpret_cast<uint64_t*>(&a)),
                                                "l"(*reinterpret_cast<uint64_t*>(&b)));
    return *reinterpret_cast<float2*>(&r);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 ng2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 ipair(float2 a) { return make_float2(-a.y, a.x); }   // i (x + i y)
__device__ __forceinline__ float2 mipair(float2 a) { return make_float2(a.y, -a.x); }  // -i (x + i y)
__device__ __forceinline__ pk pld(const float4* p)
{
    const float4 v = *p;
    return pk{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ void pst(float4* p, pk v) { *p = make_float4(v.h.x, v.h.y, v.l.x, v.l.y); }
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e)
{
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
__device__ __forceinline__ pk renorm2(float2 s, float2 e)
{
    pk r;
    r.h = add2(s, e);
    r.l = sub2(e, sub2(r.h, s));
    return r;
}
// lanes of x1 y1 + x2 y2 (x broadcast operands, y per-lane operands), double-word products exact
// to first order: the leading products p, q and their folded low-order parts ep, eq
struct prods {
    float2 p, q, ep, eq;
};
__device__ __forceinline__ prods products(float2 x1h, float2 x1l, float2 y1h, float2 y1l, float2 x2h, float2 x2l,
                                          float2 y2h, float2 y2l)
{
    prods r;
    r.p = mul2(x1h, y1h);
    r.q = mul2(x2h, y2h);
    r.ep = fma2(x1h, y1h, ng2(r.p));
    r.eq = fma2(x2h, y2h, ng2(r.q));
    r.ep = fma2(x1h, y1l, fma2(x1l, y1h, r.ep));
    r.eq = fma2(x2h, y2l, fma2(x2l, y2h, r.eq));
    return r;
}
// the double-word products of a b: lane re a.re b.re + a.im (-b.im), lane im a.re b.im + a.im b.re
__device__ __forceinline__ prods cprods(pk a, pk b)
{
    return products(bc(a.h.x), bc(a.l.x), b.h, b.l, bc(a.h.y), bc(a.l.y), ipair(b.h), ipair(b.l));
}
__device__ __forceinline__ pk cmul_pu(pk a, pk b)
{
    const prods r = cprods(a, b);
    float2 s1, t1;
    two_sum2(r.p, r.q, s1, t1);
    return pk{s1, add2(t1, add2(r.ep, r.eq))};
}
__device__ __forceinline__ pk cmul_p(pk a, pk b)
{
    const pk u = cmul_pu(a, b);
    return renorm2(u.h, u.l);
}
// a sum of two products plus z per lane: TwoSum of the leading products, TwoSum with z.hi,
// every low-order term folded once, one renormalisation
// z + a b
__device__ __forceinline__ pk dot_add(const prods& r, pk z)
{
    float2 s1, t1, s2, t2;
    two_sum2(r.p, r.q, s1, t1);
    two_sum2(s1, z.h, s2, t2);
    return renorm2(s2, add2(add2(add2(t1, t2), add2(r.ep, r.eq)), z.l));
}
__device__ __forceinline__ pk cfma_p(pk a, pk b, pk z) { return dot_add(cprods(a, b), z); }
// z - a b: lane re (-a.re) b.re + a.im b.im, lane im (-a.re) b.im + a.im (-b.re)
__device__ __forceinline__ pk cfms_p(pk a, pk b, pk z)
{
    return dot_add(products(bc(-a.h.x), bc(-a.l.x), b.h, b.l, bc(a.h.y), bc(a.l.y), mipair(b.h), mipair(b.l)), z);
}
// 10 p + a + b per lane (the Numerov right-hand side), one TwoSum per pair of leading terms,
// unnormalised (feeds a product)
__device__ __forceinline__ pk ten_sum_p(pk p, pk a, pk b)
{
    const float2 x = mul2(bc(10.f), p.h);
    const float2 ex = fma2(bc(10.f), p.l, fma2(bc(10.f), p.h, ng2(x)));
    float2 s1, t1, s2, t2;
    two_sum2(a.h, b.h, s1, t1);
    two_sum2(x, s1, s2, t2);
    return pk{s2, add2(add2(add2(t1, t2), ex), add2(a.l, b.l))};
}
// g u + y - p per lane (the CN update before the phase): the four leading terms by three
// TwoSums, every low-order term folded once, unnormalised (feeds a product)
__device__ __forceinline__ pk cn_update_p(pk g, pk u, pk y, pk p)
{
    const prods r = cprods(g, u);
    float2 s1, t1, s2, t2, s3, t3;
    two_sum2(r.p, r.q, s1, t1);
    two_sum2(y.h, ng2(p.h), s2, t2);
    two_sum2(s1, s2, s3, t3);
    return pk{s3, add2(add2(add2(t1, t2), t3), add2(add2(r.ep, r.eq), add2(y.l, ng2(p.l))))};
}
// Accumulators of a site loop: hi takes each term's leading part by a TwoSum, lo gathers every
// low-order part; renormalised once after the loop (lo stays far below ulp(hi) over a chunk).
// acc += x y per lane with x broadcast
__device__ __forceinline__ void acc_mul_p(pk& acc, float xh, float xl, pk y)
{
    const float2 X = bc(xh);
    const float2 p = mul2(X, y.h);
    float2 ep = fma2(X, y.h, ng2(p));
    ep = fma2(X, y.l, fma2(bc(xl), y.h, ep));
    float2 s, e;
    two_sum2(acc.h, p, s, e);
    acc.h = s;
    acc.l = add2(acc.l, add2(e, ep));
}
// acc += (a.re b.re + a.im b.im, a.re b.im - a.im b.re): the projection of a on b
__device__ __forceinline__ void acc_proj_p(pk& acc, pk a, pk b)
{
    const prods r = products(bc(a.h.x), bc(a.l.x), b.h, b.l, bc(a.h.y), bc(a.l.y), mipair(b.h), mipair(b.l));
    float2 s1, t1, s2, t2;
    two_sum2(r.p, r.q, s1, t1);
    two_sum2(acc.h, s1, s2, t2);
    acc.h = s2;
    acc.l = add2(acc.l, add2(add2(t1, t2), add2(r.ep, r.eq)));
}
// |v|^2, unnormalised: packed double-word squares, then the TwoSum of the two lanes
__device__ __forceinline__ df norm2_u(pk v)
{
    const float2 p = mul2(v.h, v.h);
    float2 ep = fma2(v.h, v.h, ng2(p));
    ep = fma2(v.h, v.l, fma2(v.l, v.h, ep));
    float s1, t1;
    two_sum(p.x, p.y, s1, t1);
    return df{s1, t1 + (ep.x + ep.y)};
}
__device__ __forceinline__ pk pshup(pk v, int d)
{
    return pk{make_float2(__shfl_up_sync(0xffffffffu, v.h.x, d), __shfl_up_sync(0xffffffffu, v.h.y, d)),
              make_float2(__shfl_up_sync(0xffffffffu, v.l.x, d), __shfl_up_sync(0xffffffffu, v.l.y, d))};
}
__device__ __forceinline__ pk pshdn(pk v, int d)
{
    return pk{make_float2(__shfl_down_sync(0xffffffffu, v.h.x, d), __shfl_down_sync(0xffffffffu, v.h.y, d)),
              make_float2(__shfl_down_sync(0xffffffffu, v.l.x, d), __shfl_down_sync(0xffffffffu, v.l.y, d))};
}

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

__device__ __forceinline__ df shfl_xor_df(df v, int d)
{
    return df{__shfl_xor_sync(0xffffffffu, v.hi, d), __shfl_xor_sync(0xffffffffu, v.lo, d)};
}

// exclusive CTA scans of the affine maps Y_t = b_t + c_t Y_{t-1} (forward) and
// U_t = b_t + c_t U_{t+1} (backward), as scan_forward / scan_backward (tdse_solver.cuh)
__device__ pk scan_fwd(pk c, pk b, pk* sc, pk* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const pk cp = pshup(c, d), bp = pshup(b, d);
        if (lane >= d) {
            b = cfma_p(c, bp, b);
            c = cmul_p(c, cp);
        }
    }
    if (lane == 31) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    pk yw{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int q = 0; q < w; q++) yw = cfma_p(sc[q], yw, sb[q]);
    const pk cp = pshup(c, 1), bp = pshup(b, 1);
    return lane == 0 ? yw : cfma_p(cp, yw, bp);
}

__device__ pk scan_bwd(pk c, pk b, pk* sc, pk* sb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const pk cp = pshdn(c, d), bp = pshdn(b, d);
        if (lane + d < 32) {
            b = cfma_p(c, bp, b);
            c = cmul_p(c, cp);
        }
    }
    if (lane == 0) {
        sc[w] = c;
        sb[w] = b;
    }
    __syncthreads();
    pk uw{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int q = kWarps - 1; q > w; q--) uw = cfma_p(sc[q], uw, sb[q]);
    const pk cp = pshdn(c, 1), bp = pshdn(b, 1);
    return lane == 31 ? uw : cfma_p(cp, uw, bp);
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
    __shared__ pk sc[2 * kWarps], sb[2 * kWarps];
    __shared__ double red[kWarps];
    __shared__ df redf[kWarps * 5];  // per warp: -<V'>, <x>, <psi0|psi> (re, im), window population
    // per step of the current block of kPhaseSteps: e^{i F dt x_0}, e^{i F dt dx}, e^{i F dt M dx 2^b}
    __shared__ pk s_pow[kPhaseSteps][kPhase];
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
                const df c2 = from_d(cs), s2 = from_d(sn);
                s_pow[t / kPhase][a] = pk{make_float2(c2.hi, s2.hi), make_float2(c2.lo, s2.lo)};
            }
            // ---- pass 1: local forward sweep of the right-hand side 2 M2 psi
            const pk zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
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
            pk pm = (t == 0) ? zero : pld(psi + (m - 1) * kThreads + t - 1);
            pk pc = pld(psi + t);
            pk yprev = zero;
            int su = 0;  // ring stage of the current site; the stage before it is refilled
            for (int i = 0; i < mi; i++) {
                float4* const r = my + su * kStage;
                if (i + kDepth - 1 < mi) issue1(i + kDepth - 1, my + (su == 0 ? kDepth - 1 : su - 1) * kStage);
                cp_commit();
                cp_wait<kDepth - 1>();
                const pk pn = (i + 1 < mi || t + 1 < kThreads) ? pld(r) : zero;
                const pk r2 = ten_sum_p(pc, pm, pn);
                yprev = cfms_p(pld(r + kThreads), yprev, cmul_pu(pld(r + 2 * kThreads), r2));
                pst(yl + i * kThreads + t, yprev);
                pm = pc;
                pc = pn;
                su = su + 1 == kDepth ? 0 : su + 1;
            }
            const pk yin = scan_fwd(pld(FF + (m - 1) * kThreads + t), yprev, sc, sb);
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
            pk unext = zero;
            su = 0;
            for (int j = 0; j < mi; j++) {  // site i = mi - 1 - j
                float4* const r = my + su * kStage;
                if (j + kDepth - 1 < mi) issue2(mi - kDepth - j, my + (su == 0 ? kDepth - 1 : su - 1) * kStage);
                cp_commit();
                cp_wait<kDepth - 1>();
                const pk y = cfma_p(pld(r), yin, pld(r + kThreads));
                unext = cfms_p(pld(r + 2 * kThreads), unext, y);
                pst(yl + (mi - 1 - j) * kThreads + t, unext);
                su = su + 1 == kDepth ? 0 : su + 1;
            }
            const pk uin = scan_bwd(pld(GP + t), unext, sc + kWarps, sb + kWarps);
            // ---- pass 3: backward correction, CN update, phase e^{+i F dt x}, observables
            const pk* pw = s_pow[k % kPhaseSteps];
            pk ph = pw[0];  // e^{i F dt x_0} (e^{i F dt m dx})^t = e^{i F dt x_{s0}}
#pragma unroll
            for (int b = 0; b < kPow; b++)
                if (t & (1 << b)) ph = cmul_p(ph, pw[2 + b]);
            const pk z = pw[1];
            // lanes (-<V'>, <x>) and the projection (re, im) on psi0
            pk acc01 = zero, acc23 = zero;
            df acc[5];
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
                const pk gp = pld(r), yv = pld(r + kThreads), po = pld(r + 2 * kThreads);
                // u - psi with u = G u_in + y, the CN update before the phase
                const pk d = cn_update_p(gp, uin, yv, po);
                const pk pn = cmul_p(ph, d);
                pst(psi + q, pn);
                ph = cmul_p(ph, z);
                const df n2 = norm2_u(pn);
                const pk gx = pld(r + 3 * kThreads), p0 = pld(r + 4 * kThreads);
                acc_mul_p(acc01, n2.hi, n2.lo, gx);
                acc_proj_p(acc23, pn, p0);
            }
            acc01 = renorm2(acc01.h, acc01.l);
            acc23 = renorm2(acc23.h, acc23.l);
            acc[0] = df{acc01.h.x, acc01.l.x};
            acc[1] = df{acc01.h.y, acc01.l.y};
            acc[2] = df{acc23.h.x, acc23.l.x};
            acc[3] = df{acc23.h.y, acc23.l.y};
            acc[4] = df{0.f, 0.f};  // the few sites of the population window in this chunk
            for (int64_t j = (lo > s0 ? lo : s0); j <= hi && j < s0 + m; j++) {
                const df n = norm2_u(pld(psi + (j - s0) * kThreads + t));
                acc[4] = add(acc[4], renorm(n.hi, n.lo));
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
                            const pk v = pld(psi + i * kThreads + t);
                            sp[2 * (s0 + i)] = (double)v.h.x + (double)v.l.x;
                            sp[2 * (s0 + i) + 1] = (double)v.h.y + (double)v.l.y;
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
                    const pk v = pld(psi + i * kThreads + t);
                    pf[2 * (s0 + i)] = (double)v.h.x + (double)v.l.x;
                    pf[2 * (s0 + i) + 1] = (double)v.h.y + (double)v.l.y;
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
        dst[q] = make_float4(re.hi, im.hi, re.lo, im.lo);  // the packed layout (re.hi, im.hi, re.lo, im.lo)
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
