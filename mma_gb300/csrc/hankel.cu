// hankel.cu -- far-field (Hankel) kernels: the plain FP64 form and the fast form.
//
// Reference: Hankel/Hankel_transform.py:452-519 (HankelTransform), :523-686 (Hankel_long).
// Per plane k and frequency w (k_w = w/c, D_k = distance - z_k):
//   A_k[w, r]   = pre_k(w) e^{-i k_w r^2/(2 D_k)} r S_k[w, r] wr_r      (wr = r trapezoid weights)
//   P_k[w, rho] = sum_r A_k[w, r] J0(k_w r rho / D_k)
//   FF[rho, w]  = sum_k tau_k P_k[w, rho]                               (tau = z trapezoid weights)
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

#include "../../include/mma_hankel.h"
#include "../../include/mma_tdse.h"
#include "hankel_common.cuh"
#include "s1tc.cuh"
#include "tc_sm100.cuh"

namespace mma {
namespace hk {

constexpr int kThreads = 256;
constexpr int kMaxRhoPerThread = 8;  // plain form: n_rho <= 2048
constexpr uint64_t kRingWaitNs = 2000000000ull;  // bounded waits of the ring stage 1 (2 s)

// ------------------------------------------------------------------------ plain FP64 form
// One CTA per frequency; per plane the CTA builds A_k[r] in shared memory, then each thread
// accumulates its rho values with CUDA's FP64 j0, in the reference's argument order
// k * r * rho / D.  The z-trapezoid is accumulated in registers (deterministic order).
__global__ void __launch_bounds__(kThreads) plain_kernel(mma_hankel_problem P, const double* og, const double* rg,
                                                         const double* zg, const double* rho, const void* src,
                                                         const double2* pre, double2* ff, const int64_t* slot,
                                                         double2* planes)
{
    extern __shared__ double2 A[];  // n_r
    const int64_t o = blockIdx.x;
    const int64_t Nr = P.n_r, Nz = P.n_z, Nrho = P.n_rho, No = P.n_omega;
    const double k = og[o] / kC;
    double2 acc[kMaxRhoPerThread];
#pragma unroll
    for (int q = 0; q < kMaxRhoPerThread; q++) acc[q] = make_double2(0.0, 0.0);
    for (int64_t kz = 0; kz < Nz; kz++) {
        const double D = P.distance - zg[kz];
        const double tau = trap_w(zg, kz, Nz);
        __syncthreads();
        for (int64_t r = threadIdx.x; r < Nr; r += blockDim.x) {
            const double rr = rg[r];
            const double2 s = load_src_d(src, kz * P.plane_stride + o * P.omega_stride + r, P.source_c128);
            double2 a = pre_at(P, pre, kz, o, r);  // the radial factor first, as in :505-512
            if (P.near_field) {  // exp(-1j k r^2 / (2 D)), Hankel_transform.py:506
                double sn, cs;
                sincos(-((k * (rr * rr)) / (2.0 * D)), &sn, &cs);
                a = make_double2(a.x * cs - a.y * sn, a.x * sn + a.y * cs);
            }
            a = make_double2(a.x * rr, a.y * rr);
            a = make_double2(a.x * s.x - a.y * s.y, a.x * s.y + a.y * s.x);
            const double w = trap_w(rg, r, Nr);
            A[r] = make_double2(a.x * w, a.y * w);
        }
        __syncthreads();
        const int64_t sl = slot ? slot[kz] : -1;
#pragma unroll
        for (int q = 0; q < kMaxRhoPerThread; q++) {
            const int64_t j = threadIdx.x + (int64_t)q * blockDim.x;
            if (j < Nrho) {
                const double rj = rho[j];
                double re = 0.0, im = 0.0;
                for (int64_t r = 0; r < Nr; r++) {
                    const double J = j0(k * rg[r] * rj / D);
                    re = fma(A[r].x, J, re);
                    im = fma(A[r].y, J, im);
                }
                if (sl >= 0 && planes) planes[(sl * Nrho + j) * No + o] = make_double2(re, im);
                acc[q].x = fma(tau, re, acc[q].x);
                acc[q].y = fma(tau, im, acc[q].y);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kMaxRhoPerThread; q++) {
        const int64_t j = threadIdx.x + (int64_t)q * blockDim.x;
        if (j < Nrho) ff[j * No + o] = acc[q];
    }
}

// ------------------------------------------------------------------------ fast form, stage 1
// Per-plane constants, independent of frequency, computed once per call (rows of MM + 4 floats):
//   row[m] = tau_k v_k^m (m < MM),  row[MM], row[MM+1] = 1/(2 D_k) as (hi, lo),
//   row[MM+2], row[MM+3] = 1/(2 D_k) - 1/(2 d_ref) as (hi, lo) (the plane's offset from the
//   reference distance).
template <int MM>
__global__ void fast_plane_table(mma_hankel_problem P, mma_hankel_fast_plan_t F, const double* zg, float* ptab)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < P.n_z; q += (int64_t)gridDim.x * blockDim.x) {
        const double D = P.distance - zg[q];
        const double lam = F.d_ref / D;
        const double v = (1.0 - lam * lam) / F.sigma;
        double c = trap_w(zg, q, P.n_z);
        float* row = ptab + q * (MM + 4);
        for (int m = 0; m < MM; m++) {
            row[m] = (float)c;
            c *= v;
        }
        float hi, lo;
        split_d(1.0 / (2.0 * D), hi, lo);
        row[MM] = hi;
        row[MM + 1] = lo;
        split_d(1.0 / (2.0 * D) - 1.0 / (2.0 * F.d_ref), hi, lo);
        row[MM + 2] = hi;
        row[MM + 3] = lo;
    }
}

__device__ __forceinline__ float2 f2b(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2n(float2 a) { return make_float2(-a.x, -a.y); }
// 16-byte shared-memory load kept where it stands (a volatile asm is neither hoisted out of the
// loop nor merged): the per-term tables are re-read per radius pair instead of being held in
// registers across the loop, which would spill
__device__ __forceinline__ float4 lds4(uint32_t saddr)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(saddr));
    return v;
}

// Per-frequency and per-radius constants of stage 1 as floats: ktab[w] = k_w = w/c as (hi, lo);
// rtab[r] = (r^2 as (hi, lo), trapezoid weight * r, 0).
__global__ void fast_wr_tables(mma_hankel_problem P, const double* og, const double* rg, float2* ktab, float4* rtab)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < P.n_omega; q += stride) {
        float hi, lo;
        split_d(og[q] / kC, hi, lo);
        ktab[q] = make_float2(hi, lo);
    }
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < P.n_r; q += stride) {
        const double rr = rg[q];
        float hi, lo;
        split_d(rr * rr, hi, lo);
        rtab[q] = make_float4(hi, lo, (float)(trap_w(rg, q, P.n_r) * rr), 0.f);
    }
}

// Stage 1 through a shared-memory ring, for complex64 sources whose rows start on 16-byte
// boundaries (rows of an even number of radii at even strides) and pre-factors per (plane,
// frequency).  One CTA per (frequency, 256 radii), two CTAs per SM: eight consumer warps, one
// radius per thread, and a producer warp whose lane 0 streams the source with 1-D bulk copies
// (one per plane: the plane's row of radii, 2 KB) into a ring of `ns` stages of kG planes each,
// one full and one empty mbarrier per stage, so that tens of KB per SM are in flight whatever the
// register count.  A consumer warp releases a stage as soon as it has read its values, and the
// producer refills the slot with the stage ns later once all eight have; it does no other work,
// so the refills do not wait for a consumer's arithmetic (with the producer in a consumer warp
// the kernel took 139.8 against 108.3 us on the 268 MB small_ff case).  A consumer waits once per
// stage and then accumulates its kG planes (independent chains the scheduler can interleave):
//   B_m = e^{-i k r^2 u_ref} r w_r sum_k tau_k v_k^m pre_k e^{-i delta_k} S_k,
//   delta_k = k r^2 (u_k - u_ref),  u = 1/(2 D),
// i.e. the near-field phase e^{-i k r^2 u_k} split into a per-thread reference factor, applied
// once to the finished sums together with r w_r, and the plane's offset from it.  e^{-i delta}
// comes from Taylor polynomials when every |delta| of the CTA is within 0.12, else from the
// float-float angle reduced mod 2 pi (the choice is uniform over the CTA).  The MM sums run as
// real and imaginary pairs (B_m, B_m+1) in packed FP32x2 FMAs against coefficient pairs read as
// float4 quads from shared memory; every 16 planes they are added into FP32 totals kept in
// shared memory (each thread its own column), which leaves the registers to the partial sums.
// Every wait is bounded; on a timeout the CTA stops, sets *status and writes NaN into its B values.
constexpr int kRingR = 256;  // radii per CTA, one per consumer thread
constexpr int kG = 4;        // planes per ring stage
template <int MM>
__global__ void __launch_bounds__(kRingR + 32, 2)
    fast_stage1_ring(mma_hankel_problem P, const float2* __restrict__ src, const double2* __restrict__ pre,
                     const float* __restrict__ ptab, const float2* __restrict__ ktab,
                     const float4* __restrict__ rtab, float2 u_ref, float2* Bp, int ns, int* status, int no_issue)
{
    static_assert(MM % 4 == 0 && MM <= 16, "ring stage 1 takes 4, 8, 12 or 16 terms");
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ unsigned s_dumax;
    constexpr int RW = MM + 4;
    constexpr int MQ = MM / 4;  // coefficient quads per plane
    const int Nz = (int)P.n_z;
    const int64_t o = blockIdx.y, Nr = P.n_r, No = P.n_omega;
    const int64_t r0 = (int64_t)blockIdx.x * kRingR;
    const int cnt = (int)(Nr - r0 < kRingR ? Nr - r0 : kRingR);
    const int n_st = (Nz + kG - 1) / kG;  // stages of planes, the last possibly partial
    float2* ring = reinterpret_cast<float2*>(smem_raw);                        // ns x kG x kRingR values
    float4* tots = reinterpret_cast<float4*>(ring + (size_t)ns * kG * kRingR);  // 2 MQ x kRingR: re, im quads
    float4* coef = tots + 2 * MQ * kRingR;                                     // Nz x MQ: c_4q .. c_4q+3
    float4* pinfo = coef + Nz * MQ;                                            // Nz: (pre re, pre im, du hi, du lo)
    uint64_t* full = reinterpret_cast<uint64_t*>(pinfo + Nz);
    uint64_t* empty = full + ns;
    volatile int* abort_s = reinterpret_cast<volatile int*>(empty + ns);
    const int t = threadIdx.x, lane = t & 31;
    const uint32_t bytes = (uint32_t)cnt * 8u;
    const float2* row0 = src + o * P.omega_stride + r0;
    // issue stage j (planes j kG ...) into ring slot `slot`: one copy per plane, one barrier
    auto issue = [&](int j, int slot) {
        const int k0 = j * kG, np = Nz - k0 < kG ? Nz - k0 : kG;
        tc::mbar_arrive_expect_tx(&full[slot], bytes * (uint32_t)np);
        for (int g = 0; g < np; g++)
            tc::bulk_load_1d(ring + ((size_t)slot * kG + g) * kRingR, row0 + (int64_t)(k0 + g) * P.plane_stride,
                             bytes, &full[slot]);
    };
    if (t == 0) {
        for (int q = 0; q < ns; q++) {
            tc::mbar_init(&full[q], 1);
            tc::mbar_init(&empty[q], kRingR / 32);
        }
        *abort_s = 0;
        s_dumax = 0u;
        tc::fence_barrier_init();
        if (!no_issue)  // (no_issue: the test of the bounded waits, nothing is ever copied)
            for (int j = 0; j < n_st && j < ns; j++) issue(j, j);  // the first stages, before the tables
    }
    for (int q = t; q < Nz * MQ; q += blockDim.x) {
        const float* row = ptab + (q / MQ) * RW + (q % MQ) * 4;
        coef[q] = make_float4(row[0], row[1], row[2], row[3]);
    }
    if (t < kRingR)
#pragma unroll
        for (int q = 0; q < 2 * MQ; q++) tots[q * kRingR + t] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();  // s_dumax initialised
    {
        unsigned mx = 0u;  // max |u_k - u_ref| as float bits (non-negative floats order as integers)
        for (int q = t; q < Nz; q += blockDim.x) {
            const double2 pf = pre ? pre[q * No + o] : make_double2(1.0, 0.0);
            const float duh = ptab[q * RW + MM + 2], dul = ptab[q * RW + MM + 3];
            pinfo[q] = make_float4((float)pf.x, (float)pf.y, duh, dul);
            mx = max(mx, __float_as_uint(fabsf(duh)));
        }
        atomicMax(&s_dumax, mx);
    }
    __syncthreads();
    int issued = no_issue ? 0 : (n_st < ns ? n_st : ns);  // stages issued: the first ns by thread 0, then the producer
    // ---------------------------------------------------------------- per-thread constants
    const bool active = t < cnt;
    const int64_t r = r0 + (active ? t : 0);
    const float2 kk = ktab[o];
    const float4 rt = rtab[r];
    // k r^2 as float-float
    const float kr2h = kk.x * rt.x;
    const float kr2l = fmaf(kk.x, rt.x, -kr2h) + fmaf(kk.x, rt.y, kk.y * rt.x);
    const bool near = P.near_field != 0;
    // near-field mode, uniform over the CTA: 0 none, 1 small angles, 2 exact reduction per element
    const bool small = __syncthreads_and(fabsf(kr2h) * __uint_as_float(s_dumax) <= 0.12f);
    const int mode = !near ? 0 : (small ? 1 : 2);
    // partial sums of the current 16 planes: pr[j] = (Re B_2j, Re B_2j+1), pi[j] likewise imaginary
    float2 pr[MM / 2], pim[MM / 2];
#pragma unroll
    for (int q = 0; q < MM / 2; q++) pr[q] = pim[q] = make_float2(0.f, 0.f);
    // one plane: a = pre S e^{-i delta}, then the MM partial sums
    auto plane = [&](const float2 sv, const int kz, const int md) {
        const float4 pf = pinfo[kz];
        // pre S as a packed pair: lane re pre.re S.re + pre.im (-S.im), lane im pre.re S.im + pre.im S.re
        float2 a = __ffma2_rn(f2b(pf.x), sv, __fmul2_rn(f2b(pf.y), make_float2(-sv.y, sv.x)));
        if (md != 0) {
            float sn, cs;
            if (md == 1) {
                sincos_small_p(kr2h * pf.z, sn, cs);
            } else {  // the angle k r^2 (u_k - u_ref) in float-float, reduced mod 2 pi
                const float th = kr2h * pf.z;
                const float te = fmaf(kr2h, pf.z, -th) + fmaf(kr2h, pf.w, kr2l * pf.z);
                sincos_reduced(reduce_2pi(th, te), sn, cs);
            }
            // a e^{-i delta}: lane re a.re cs + sn a.im, lane im a.im cs + sn (-a.re)
            a = __ffma2_rn(a, f2b(cs), __fmul2_rn(f2b(sn), make_float2(a.y, -a.x)));
        }
        const float2 ax = make_float2(a.x, a.x), ay = make_float2(a.y, a.y);
        const float4* c4 = coef + kz * MQ;
#pragma unroll
        for (int q = 0; q < MQ; q++) {
            const float4 c = c4[q];
            pr[2 * q] = __ffma2_rn(make_float2(c.x, c.y), ax, pr[2 * q]);
            pr[2 * q + 1] = __ffma2_rn(make_float2(c.z, c.w), ax, pr[2 * q + 1]);
            pim[2 * q] = __ffma2_rn(make_float2(c.x, c.y), ay, pim[2 * q]);
            pim[2 * q + 1] = __ffma2_rn(make_float2(c.z, c.w), ay, pim[2 * q + 1]);
        }
    };
    bool ok = true;
    if (t >= kRingR) {
        // the producer warp: lane 0 refills each slot with the stage ns later as soon as every
        // consumer warp has released it, then waits until its last copies have landed (on an abort
        // too: the ring must outlive the copies in flight)
        if (lane == 0) {
            int sp = 0;
            uint32_t php = 0;
            for (int jj = no_issue ? n_st : issued; jj < n_st; jj++) {
                if (!tc::mbar_wait_spin(&empty[sp], php, abort_s, kRingWaitNs)) {
                    if (!*abort_s) {
                        *abort_s = 1;
                        atomicCAS(status, 0, 1);
                    }
                    break;
                }
                issue(jj, sp);
                issued = jj + 1;
                if (++sp == ns) {
                    sp = 0;
                    php ^= 1u;
                }
            }
            for (int j = (issued > ns ? issued - ns : 0); j < issued; j++)
                tc::mbar_wait(&full[j % ns], (uint32_t)(j / ns) & 1u, nullptr, kRingWaitNs);
        }
        return;
    }
    // ring slot and phase parity of stage j, counted incrementally (no divisions)
    int s = 0;
    uint32_t ph = 0;
    // add the 16-plane partial sums into the totals
    auto flush = [&]() {
#pragma unroll
        for (int q = 0; q < MQ; q++) {
            float4* tr = tots + (2 * q) * kRingR + t;
            float4* ti = tots + (2 * q + 1) * kRingR + t;
            float4 vr = *tr, vi = *ti;
            const float2 r01 = __fadd2_rn(make_float2(vr.x, vr.y), pr[2 * q]);
            const float2 r23 = __fadd2_rn(make_float2(vr.z, vr.w), pr[2 * q + 1]);
            const float2 i01 = __fadd2_rn(make_float2(vi.x, vi.y), pim[2 * q]);
            const float2 i23 = __fadd2_rn(make_float2(vi.z, vi.w), pim[2 * q + 1]);
            *tr = make_float4(r01.x, r01.y, r23.x, r23.y);
            *ti = make_float4(i01.x, i01.y, i23.x, i23.y);
            pr[2 * q] = pr[2 * q + 1] = pim[2 * q] = pim[2 * q + 1] = make_float2(0.f, 0.f);
        }
    };
    // wait for stage j's slot, read this thread's kG values and release the slot
    auto take = [&](float2 (&sv)[kG]) -> bool {
        if (!tc::mbar_wait_spin(&full[s], ph, abort_s, kRingWaitNs)) {
            *abort_s = 1;
            atomicCAS(status, 0, 2);
            return false;
        }
#pragma unroll
        for (int g = 0; g < kG; g++) sv[g] = ring[(s * kG + g) * kRingR + t];  // rows beyond cnt: unused
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&empty[s]);
        if (++s == ns) {
            s = 0;
            ph ^= 1u;
        }
        return true;
    };
    constexpr int kGroup = 16 / kG;  // stages per 16 planes
    int j = 0;
    // the common case, small near-field angles: groups of kGroup full stages, kG independent chains
    // per stage and the totals updated after each group, with no per-stage tests
    const int n_grp = mode == 1 ? Nz / 16 : 0;
    for (int gi = 0; gi < n_grp && ok; gi++) {
#pragma unroll
        for (int u = 0; u < kGroup; u++) {
            float2 sv[kG];
            if (!take(sv)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int g = 0; g < kG; g++) plane(sv[g], (j + u) * kG + g, 1);
        }
        j += kGroup;
        if (ok) flush();
    }
    // the rest: no near field, exact angles, and the last planes (static indices keep sv in registers)
    for (; ok && j < n_st; j++) {
        float2 sv[kG];
        if (!take(sv)) {
            ok = false;
            break;
        }
        const int k0 = j * kG;
#pragma unroll
        for (int g = 0; g < kG; g++)
            if (k0 + g < Nz) plane(sv[g], k0 + g, mode);
        if (j % kGroup == kGroup - 1 || j == n_st - 1) flush();
    }
    if (!active) return;
    // the per-thread factor r w_r e^{-i k r^2 u_ref}
    float2 bw = make_float2(rt.z, 0.f);
    if (near) {
        const float th = kr2h * u_ref.x;
        const float te = fmaf(kr2h, u_ref.x, -th) + fmaf(kr2h, u_ref.y, kr2l * u_ref.x);
        float sn, cs;
        sincos_reduced(reduce_2pi(th, te), sn, cs);
        bw = make_float2(rt.z * cs, -rt.z * sn);
    }
    const float nan = __int_as_float(0x7fc00000);
#pragma unroll
    for (int q = 0; q < MQ; q++) {
        const float4 vr = tots[(2 * q) * kRingR + t], vi = tots[(2 * q + 1) * kRingR + t];
        const float re[4] = {vr.x, vr.y, vr.z, vr.w}, im[4] = {vi.x, vi.y, vi.z, vi.w};
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float2 b = make_float2(fmaf(bw.x, re[u], -bw.y * im[u]), fmaf(bw.x, im[u], bw.y * re[u]));
            Bp[(o * MM + 4 * q + u) * Nr + r] = ok ? b : make_float2(nan, nan);
        }
    }
}

// z-contraction B_m[w, r] = sum_k tau_k v_k^m A_k[w, r]: one thread per (w, r), source read once,
// four planes in flight per thread.
template <int MM>
__global__ void __launch_bounds__(kThreads) fast_stage1(mma_hankel_problem P, const double* og, const double* rg,
                                                        const void* src, const double2* pre, const float* ptab,
                                                        float2* Bp)
{
    extern __shared__ float smem[];
    const int64_t o = blockIdx.y, Nz = P.n_z, Nr = P.n_r, No = P.n_omega;
    constexpr int RW = MM + 4;
    float* tabs = smem;                                                   // Nz * RW
    float2* pr = reinterpret_cast<float2*>(smem + ((Nz * RW + 1) / 2) * 2);  // Nz: pre-factor
    for (int64_t q = threadIdx.x; q < Nz * RW; q += blockDim.x) tabs[q] = ptab[q];
    for (int64_t q = threadIdx.x; q < Nz; q += blockDim.x) {
        const double2 pf = (pre && !P.pre_radial) ? pre[q * No + o] : make_double2(1.0, 0.0);
        pr[q] = make_float2((float)pf.x, (float)pf.y);
    }
    __syncthreads();
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= Nr) return;  // no barrier below
    float kh, kl;  // k_w as float-float
    split_d(og[o] / kC, kh, kl);
    const double rr = rg[r];
    float r2h, r2l;
    split_d(rr * rr, r2h, r2l);
    // k r^2 as float-float; the plane angle is (k r^2) * (1/(2 D_k))
    const float kr2h = kh * r2h;
    const float kr2l = fmaf(kh, r2h, -kr2h) + fmaf(kh, r2l, kl * r2h);
    const float wr = (float)(trap_w(rg, r, Nr) * rr);
    float2 part[MM], hi[MM], lo[MM];
#pragma unroll
    for (int m = 0; m < MM; m++) part[m] = hi[m] = lo[m] = make_float2(0.f, 0.f);
    const int64_t base = o * P.omega_stride + r;
    for (int64_t k0 = 0; k0 < Nz; k0 += 4) {
        float2 sv[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            sv[u] = (k0 + u < Nz) ? load_src_f(src, (k0 + u) * P.plane_stride + base, P.source_c128)
                                  : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t kz = k0 + u;
            if (kz >= Nz) break;
            const float* row = tabs + kz * RW;
            float2 pf = pr[kz];
            if (P.pre_radial) {
                const double2 pd = pre_at(P, pre, kz, o, r);
                pf = make_float2((float)pd.x, (float)pd.y);
            }
            float2 a = make_float2(fmaf(pf.x, sv[u].x, -pf.y * sv[u].y), fmaf(pf.x, sv[u].y, pf.y * sv[u].x));
            if (P.near_field) {
                const float ih = row[MM], il = row[MM + 1];
                const float th = kr2h * ih;
                const float te = fmaf(kr2h, ih, -th) + fmaf(kr2h, il, kr2l * ih);
                float sn, cs;
                sincos_reduced(reduce_2pi(th, te), sn, cs);  // e^{-i theta} = (cs, -sn)
                a = make_float2(fmaf(a.x, cs, a.y * sn), fmaf(a.y, cs, -a.x * sn));
            }
            a.x *= wr;
            a.y *= wr;
#pragma unroll
            for (int m = 0; m < MM; m++) {
                part[m].x = fmaf(row[m], a.x, part[m].x);
                part[m].y = fmaf(row[m], a.y, part[m].y);
            }
            if ((kz & 15) == 15 || kz == Nz - 1) {
#pragma unroll
                for (int m = 0; m < MM; m++) {
                    ff_acc(hi[m].x, lo[m].x, part[m].x);
                    ff_acc(hi[m].y, lo[m].y, part[m].y);
                    part[m] = make_float2(0.f, 0.f);
                }
            }
        }
    }
#pragma unroll
    for (int m = 0; m < MM; m++) Bp[(o * MM + m) * Nr + r] = make_float2(hi[m].x + lo[m].x, hi[m].y + lo[m].y);
}

// ------------------------------------------------------------------------ fast form, stage 2
// FF[rho, w] = sum_r sum_m K_m(y) B_m[w, r], y = k_w r rho / d_ref, with
//   K_0 = J0(y), K_1 = (sigma y/2) J1(y),
//   K_{m+1} = sigma m/(m+1) K_m - (sigma y/2)^2 / (m (m+1)) K_{m-1}
// (J_{m+1} = (2m/y) J_m - J_{m-1} rescaled by (sigma y/2)^m/m!: no division by y).
// One thread per (w, rho); B and k r / d_ref staged in shared memory in tiles of r.
// With SER the same K_m(y) also give up to kSeriesPlanes single planes, the fast form's entry and
// exit planes: P_k[rho, w] = sum_r A_k[w, r] sum_m v_k^m K_m(y) (J0(lambda_k y) by the same
// series), with A_k from series_plane_a and the pairs (v_k0^m, v_k1^m) from series_plane_tables;
// the planes' sums run as FP32x2 pairs (one lane per plane) beside the far field's.
constexpr int kSeriesPlanes = 2;
template <int MM, bool SER>
__global__ void __launch_bounds__(kThreads, SER ? 2 : 3) fast_stage2(mma_hankel_problem P, mma_hankel_fast_plan_t F,
                                                        const double* og, const double* rg, const double* rho,
                                                        const float2* Bp, double2* ff, int rtile,
                                                        const float2* asel, const float2* vsel, int n_sel,
                                                        double2* planes, float x_cut8, float x_cut4)
{
    extern __shared__ __align__(16) float smem[];
    const int64_t o = blockIdx.y, Nr = P.n_r, Nrho = P.n_rho, No = P.n_omega;
    // B_m of the tile's radius pairs: row m, pair p = (Re B_m[2p], Re B_m[2p+1], Im B_m[2p], Im B_m[2p+1])
    float4* B4 = reinterpret_cast<float4*>(smem);  // MM * rtile / 2 (rtile even)
    float2* kr = reinterpret_cast<float2*>(B4 + MM * (rtile / 2));  // rtile
    float2* As = kr + rtile;                       // SER: kSeriesPlanes * rtile, A_k of the selected planes
    float2* Vs = As + kSeriesPlanes * rtile;       // SER: MM pairs (v_k0^m, v_k1^m)
    // per term m the recurrence's constants as broadcast pairs (s m/(m+1), -1/(m(m+1))) and, with
    // SER, the planes' (v_k0^m, v_k1^m) as broadcast pairs: read whole by one 16-byte load
    float4* Cm = reinterpret_cast<float4*>(kr + rtile + (SER ? kSeriesPlanes * rtile + MM : 0));
    float4* Vb = Cm + MM;  // SER
    const uint32_t cm_s = (uint32_t)__cvta_generic_to_shared(Cm), vb_s = cm_s + 16u * MM;
    const float s = (float)F.sigma;
    for (int m = threadIdx.x; m < MM; m += blockDim.x) {
        const float c1 = s * __fdiv_rn((float)m, (float)(m + 1));
        const float c2 = m > 0 ? -__fdiv_rn(1.0f, (float)(m * (m + 1))) : 0.f;
        Cm[m] = make_float4(c1, c1, c2, c2);
        if (SER) {
            const float2 v = vsel[m];
            Vs[m] = v;
            Vb[m] = make_float4(v.x, v.x, v.y, v.y);
        }
    }
    float2 ppart[kSeriesPlanes], phi[kSeriesPlanes], plo[kSeriesPlanes];  // the planes' compensated sums
#pragma unroll
    for (int i = 0; i < kSeriesPlanes; i++) ppart[i] = phi[i] = plo[i] = make_float2(0.f, 0.f);
    const double kap = (og[o] / kC) / F.d_ref;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float rh = 0.f, rl = 0.f;
    if (j < Nrho) split_d(rho[j], rh, rl);
    // the series length per (warp, chunk of kChunk radii): sigma y / 2 <= x_cut8 (x_cut4) lets MM - 8
    // (MM - 4) terms meet the plan's truncation bound, y <= (k r / d_ref)_max of the chunk times
    // the warp's largest rho
    constexpr int kChunk = 32;
    __shared__ float s_krm[64];  // per chunk of the tile: the largest k r / d_ref
    const float rho_w = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(rh))));
    float2 part = make_float2(0.f, 0.f), hi = part, lo = part;
    int cnt = 0;
    for (int64_t r0 = 0; r0 < Nr; r0 += rtile) {
        const int64_t nt = (Nr - r0 < rtile) ? (Nr - r0) : rtile;
        __syncthreads();
        for (int64_t q = threadIdx.x; q < MM * nt; q += blockDim.x) {
            const int64_t m = q / nt, rr = q % nt;
            const float2 v = Bp[(o * MM + m) * Nr + r0 + rr];
            float* w = reinterpret_cast<float*>(B4 + m * (rtile / 2) + rr / 2) + (rr & 1);
            w[0] = v.x;
            w[2] = v.y;
        }
        for (int64_t q = threadIdx.x; q < nt; q += blockDim.x) {
            float h, l;
            split_d(kap * rg[r0 + q], h, l);
            kr[q] = make_float2(h, l);
            if (SER)
#pragma unroll
                for (int i = 0; i < kSeriesPlanes; i++) As[i * rtile + q] = asel[((int64_t)i * No + o) * Nr + r0 + q];
        }
        __syncthreads();
        if (threadIdx.x < (nt + kChunk - 1) / kChunk) {
            const int64_t c0 = threadIdx.x * kChunk, c1 = c0 + kChunk < nt ? c0 + kChunk : nt;
            float mx = 0.f;
            for (int64_t q = c0; q < c1; q++) mx = fmaxf(mx, fabsf(kr[q].x));
            s_krm[threadIdx.x] = mx * 1.000001f;  // k r / d_ref's low part and rounding: a hair above
        }
        __syncthreads();
        if (j < Nrho) {
            // radius pairs: each per-radius quantity is a pair, so the y products, K_1, the
            // m-recurrence and the contraction run as packed FP32x2 instructions (each lane the
            // single-radius operations in the same order); the two radii's J0/J1 seeds are
            // independent chains the scheduler interleaves.  The row stride rtile is even, so a
            // pair's B values and k r / d_ref entries are one 16-byte load each.
            const float4* kr4 = reinterpret_cast<const float4*>(kr);
            // one radius's terms: the far field's, and with SER the planes' A_k[r] sum_m v_k^m K_m
            auto add_in = [&](float2 in, int64_t q, float2 sv) {
                part = __fadd2_rn(part, in);
                if (SER) {
                    ppart[0] = __ffma2_rn(As[q], f2b(sv.x), ppart[0]);
                    ppart[1] = __ffma2_rn(As[rtile + q], f2b(sv.y), ppart[1]);
                }
                if (++cnt == 16) {
                    ff_acc(hi.x, lo.x, part.x);
                    ff_acc(hi.y, lo.y, part.y);
                    part = make_float2(0.f, 0.f);
                    if (SER)
#pragma unroll
                        for (int i = 0; i < kSeriesPlanes; i++) {
                            ff_acc(phi[i].x, plo[i].x, ppart[i].x);
                            ff_acc(phi[i].y, plo[i].y, ppart[i].y);
                            ppart[i] = make_float2(0.f, 0.f);
                        }
                    cnt = 0;
                }
            };
            // radius pairs q, q + 1 in [qa, qb) with ML series terms
            auto pairs = [&](auto MLc, int64_t qa, int64_t qb) {
              constexpr int ML = decltype(MLc)::value;
              for (int64_t q = qa; q + 1 < qb; q += 2) {
                const float4 kk = kr4[q / 2];
                const float2 kh = make_float2(kk.x, kk.z), kl = make_float2(kk.y, kk.w);
                const float2 yh = __fmul2_rn(kh, f2b(rh));
                const float2 yl = __fadd2_rn(__ffma2_rn(kh, f2b(rh), f2n(yh)), __ffma2_rn(kh, f2b(rl), __fmul2_rn(kl, f2b(rh))));
                float2 J0, J1;
                bessel01x2<true>(yh, yl, J0, J1);
                const float2 y = __fadd2_rn(yh, yl);
                float2 K0 = J0;
                float2 K1 = __fmul2_rn(__fmul2_rn(f2b(0.5f * s), y), J1);
                const float2 q2 = __fmul2_rn(__fmul2_rn(f2b(0.25f * s * s), y), y);
                // lanes = the two radii throughout: the real and the imaginary parts of the far
                // field's sum, and (SER) the planes' sums sum_m v_k0^m K_m and sum_m v_k1^m K_m
                const float4 b0 = B4[q / 2], b1 = B4[rtile / 2 + q / 2];
                float2 sre = __ffma2_rn(make_float2(b0.x, b0.y), K0, __fmul2_rn(make_float2(b1.x, b1.y), K1));
                float2 sim = __ffma2_rn(make_float2(b0.z, b0.w), K0, __fmul2_rn(make_float2(b1.z, b1.w), K1));
                float2 s0 = make_float2(0.f, 0.f), s1 = s0;
                if (SER) {
                    const float4 v = lds4(vb_s + 16u);
                    s0 = __ffma2_rn(make_float2(v.x, v.y), K1, K0);  // v^0 = 1
                    s1 = __ffma2_rn(make_float2(v.z, v.w), K1, K0);
                }
#pragma unroll
                for (int m = 1; m + 1 < ML; m++) {
                    const float4 c = lds4(cm_s + 16u * m);
                    const float2 K2 = __ffma2_rn(make_float2(c.x, c.y), K1,
                                                 __fmul2_rn(__fmul2_rn(q2, make_float2(c.z, c.w)), K0));
                    const float4 b = B4[(m + 1) * (rtile / 2) + q / 2];
                    sre = __ffma2_rn(make_float2(b.x, b.y), K2, sre);
                    sim = __ffma2_rn(make_float2(b.z, b.w), K2, sim);
                    if (SER) {
                        const float4 v = lds4(vb_s + 16u * (m + 1));
                        s0 = __ffma2_rn(make_float2(v.x, v.y), K2, s0);
                        s1 = __ffma2_rn(make_float2(v.z, v.w), K2, s1);
                    }
                    K0 = K1;
                    K1 = K2;
                }
                add_in(make_float2(sre.x, sim.x), q, make_float2(s0.x, s1.x));
                add_in(make_float2(sre.y, sim.y), q + 1, make_float2(s0.y, s1.y));
              }
            };
            const float hs = 0.5f * s * rho_w;
            for (int64_t c0 = 0; c0 + 1 < nt; c0 += kChunk) {
                const int64_t c1 = c0 + kChunk < nt ? c0 + kChunk : nt;
                const float xc = hs * s_krm[c0 / kChunk];  // warp-uniform
                if (MM > 8 && xc <= x_cut8)
                    pairs(std::integral_constant<int, (MM > 8 ? MM - 8 : MM)>{}, c0, c1);
                else if (MM > 4 && xc <= x_cut4)
                    pairs(std::integral_constant<int, (MM > 4 ? MM - 4 : MM)>{}, c0, c1);
                else
                    pairs(std::integral_constant<int, MM>{}, c0, c1);
            }
            const int64_t q = nt - 1;
            if (nt & 1) {  // an odd last radius (all MM terms)
                const float2 kk = kr[q];
                const float yh = kk.x * rh;
                const float yl = fmaf(kk.x, rh, -yh) + fmaf(kk.x, rl, kk.y * rh);
                float J0, J1;
                bessel01<true>(yh, yl, J0, J1);
                const float y = yh + yl;
                float K0 = J0, K1 = 0.5f * s * y * J1;
                const float q2 = 0.25f * s * s * y * y;
                const float* bq = reinterpret_cast<const float*>(B4 + q / 2) + (q & 1);  // row m at + 2 m rtile
                float2 in = make_float2(fmaf(bq[0], K0, bq[2 * rtile] * K1), fmaf(bq[2], K0, bq[2 * rtile + 2] * K1));
                float2 sa = make_float2(0.f, 0.f);
                if (SER) sa = __ffma2_rn(Vs[1], f2b(K1), f2b(K0));
#pragma unroll
                for (int m = 1; m + 1 < MM; m++) {
                    const float K2 = fmaf(s * ((float)m / (float)(m + 1)), K1, -(q2 * (1.0f / (float)(m * (m + 1)))) * K0);
                    in.x = fmaf(bq[(m + 1) * 2 * rtile], K2, in.x);
                    in.y = fmaf(bq[(m + 1) * 2 * rtile + 2], K2, in.y);
                    if (SER) sa = __ffma2_rn(Vs[m + 1], f2b(K2), sa);
                    K0 = K1;
                    K1 = K2;
                }
                add_in(in, q, sa);
            }
        }
    }
    if (j < Nrho) {
        ff_acc(hi.x, lo.x, part.x);
        ff_acc(hi.y, lo.y, part.y);
        ff[j * No + o] = make_double2((double)hi.x + (double)lo.x, (double)hi.y + (double)lo.y);
        if (SER)
#pragma unroll
            for (int i = 0; i < kSeriesPlanes; i++) {
                ff_acc(phi[i].x, plo[i].x, ppart[i].x);
                ff_acc(phi[i].y, plo[i].y, ppart[i].y);
                if (i < n_sel)
                    planes[((int64_t)i * Nrho + j) * No + o] =
                        make_double2((double)phi[i].x + (double)plo[i].x, (double)phi[i].y + (double)plo[i].y);
            }
    }
}

// Tables of the planes that stage 2 evaluates by the series: for output slot i < n_sel the plane
// k with slot[k] == i (slot i >= n_sel repeats slot 0), sel_kz[i] = k and, per term m,
// vsel[m] = (v_k0^m, v_k1^m), v_k = (1 - lambda_k^2) / sigma (in FP64, rounded once).
__global__ void series_plane_tables(mma_hankel_problem P, mma_hankel_fast_plan_t F, const double* zg,
                                    const int64_t* slot, int n_sel, int mm, int* sel_kz, float2* vsel)
{
    __shared__ int s_kz[kSeriesPlanes];  // the last plane holding each slot (0 if none)
    __shared__ double s_v[kSeriesPlanes];
    if (threadIdx.x < kSeriesPlanes) s_kz[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t q = threadIdx.x; q < P.n_z; q += blockDim.x) {
        const int64_t sl = slot[q];
#pragma unroll
        for (int i = 0; i < kSeriesPlanes; i++)
            if (sl == (i < n_sel ? i : 0)) atomicMax(&s_kz[i], (int)q);
    }
    __syncthreads();
    if (threadIdx.x < kSeriesPlanes) {
        const int i = threadIdx.x, kz = s_kz[i];
        sel_kz[i] = kz;
        const double lam = F.d_ref / (P.distance - zg[kz]);
        s_v[i] = (1.0 - lam * lam) / F.sigma;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < mm; m += blockDim.x) {
        double c0 = 1.0, c1 = 1.0;
        for (int q = 0; q < m; q++) {
            c0 *= s_v[0];
            c1 *= s_v[1];
        }
        vsel[m] = make_float2((float)c0, (float)c1);
    }
}

// A_k[w, r] = pre_k(w) e^{-i k r^2/(2 D_k)} r w_r S_k[w, r] of the series planes, in FP32 with the
// phase angle as float-float (k r^2 from ktab and rtab, 1/(2 D_k) from the plane table) reduced
// mod 2 pi: asel[i][w][r].  Grid (radius blocks, frequencies, kSeriesPlanes).
template <int MM>
__global__ void series_plane_a(mma_hankel_problem P, const float2* ktab, const float4* rtab, const float* ptab,
                              const void* src, const double2* pre, const int* sel_kz, float2* asel)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, o = blockIdx.y, i = blockIdx.z;
    if (r >= P.n_r) return;
    const int64_t kz = sel_kz[i];
    const double2 pd = pre_at(P, pre, kz, o, r);
    const float2 sv = load_src_f(src, kz * P.plane_stride + o * P.omega_stride + r, P.source_c128);
    const float2 pf = make_float2((float)pd.x, (float)pd.y);
    float2 a = make_float2(fmaf(pf.x, sv.x, -pf.y * sv.y), fmaf(pf.x, sv.y, pf.y * sv.x));
    const float4 rt = rtab[r];
    if (P.near_field) {
        const float2 kk = ktab[o];
        const float kr2h = kk.x * rt.x;
        const float kr2l = fmaf(kk.x, rt.x, -kr2h) + fmaf(kk.x, rt.y, kk.y * rt.x);
        const float ih = ptab[kz * (MM + 4) + MM], il = ptab[kz * (MM + 4) + MM + 1];
        const float th = kr2h * ih;
        const float te = fmaf(kr2h, ih, -th) + fmaf(kr2h, il, kr2l * ih);
        float sn, cs;
        sincos_reduced(reduce_2pi(th, te), sn, cs);  // e^{-i theta} = (cs, -sn)
        a = make_float2(fmaf(a.x, cs, a.y * sn), fmaf(a.y, cs, -a.x * sn));
    }
    asel[(i * P.n_omega + o) * P.n_r + r] = make_float2(a.x * rt.z, a.y * rt.z);
}

// ------------------------------------------------------------------------ fast form, single planes
// P_k[w, rho] evaluated directly in FP32 (one J0 per term): grid (rho blocks, w, requested plane).
__global__ void __launch_bounds__(kThreads) fast_planes(mma_hankel_problem P, const double* og, const double* rg,
                                                        const double* zg, const double* rho, const void* src,
                                                        const double2* pre, const int64_t* slot, double2* planes,
                                                        int rtile)
{
    extern __shared__ float smem[];
    float2* A = reinterpret_cast<float2*>(smem);  // rtile
    float2* kd = A + rtile;                       // rtile: k r / D_k (hi, lo)
    const int64_t o = blockIdx.y, Nr = P.n_r, Nrho = P.n_rho, No = P.n_omega, Nz = P.n_z;
    const int64_t want = blockIdx.z;
    int64_t kz = -1;
    for (int64_t q = 0; q < Nz; q++)
        if (slot[q] == want) kz = q;
    if (kz < 0) return;  // uniform over the CTA
    const double k = og[o] / kC, D = P.distance - zg[kz];
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float rh = 0.f, rl = 0.f;
    if (j < Nrho) split_d(rho[j], rh, rl);
    float2 part = make_float2(0.f, 0.f), hi = part, lo = part;
    int cnt = 0;
    for (int64_t r0 = 0; r0 < Nr; r0 += rtile) {
        const int64_t nt = (Nr - r0 < rtile) ? (Nr - r0) : rtile;
        __syncthreads();
        for (int64_t q = threadIdx.x; q < nt; q += blockDim.x) {
            const int64_t r = r0 + q;
            const double rr = rg[r];
            const double2 sd = load_src_d(src, kz * P.plane_stride + o * P.omega_stride + r, P.source_c128);
            double2 a = pre_at(P, pre, kz, o, r);
            if (P.near_field) {
                double sn, cs;
                sincos(-((k * (rr * rr)) / (2.0 * D)), &sn, &cs);
                a = make_double2(a.x * cs - a.y * sn, a.x * sn + a.y * cs);
            }
            const double w = trap_w(rg, r, Nr) * rr;
            a = make_double2(a.x * w, a.y * w);
            A[q] = make_float2((float)(a.x * sd.x - a.y * sd.y), (float)(a.x * sd.y + a.y * sd.x));
            float h, l;
            split_d(k * rr / D, h, l);
            kd[q] = make_float2(h, l);
        }
        __syncthreads();
        if (j < Nrho) {
            for (int64_t q = 0; q < nt; q++) {
                const float2 kk = kd[q];
                const float yh = kk.x * rh;
                const float yl = fmaf(kk.x, rh, -yh) + fmaf(kk.x, rl, kk.y * rh);
                float J0, J1;
                bessel01<false>(yh, yl, J0, J1);
                part.x = fmaf(A[q].x, J0, part.x);
                part.y = fmaf(A[q].y, J0, part.y);
                if (++cnt == 16) {
                    ff_acc(hi.x, lo.x, part.x);
                    ff_acc(hi.y, lo.y, part.y);
                    part = make_float2(0.f, 0.f);
                    cnt = 0;
                }
            }
        }
    }
    if (j < Nrho) {
        ff_acc(hi.x, lo.x, part.x);
        ff_acc(hi.y, lo.y, part.y);
        planes[(want * Nrho + j) * No + o] = make_double2((double)hi.x + (double)lo.x, (double)hi.y + (double)lo.y);
    }
}


constexpr int kTerms[] = {8, 12, 16, 20, 24, 32, 40, 48};

}  // namespace hk
}  // namespace mma

using namespace mma::hk;

// Stage 1 of the fast form: 1 (default) = the CUDA-core ring; 0 = on the tensor cores where it
// applies (16 terms, complex64 rows on 16-byte boundaries), else the CUDA-core ring.  The
// tensor-core form measured slower and less accurate on config 3 (TF32 split precision, N = 16
// MMAs that keep the tensor pipe about 20% busy), so it is not the default.
static int g_stage1_mode = 1;
// Test of the ring's bounded waits: when set, the ring's copies are never issued (every wait of
// the call runs out after kRingWaitNs; the far field is NaN and the status word reports it).
static int g_ring_no_issue = 0;

extern "C" int mma_hankel_plain(const mma_hankel_problem* p, const double* ogrid, const double* rgrid,
                                const double* zgrid, const double* rho, const void* source, const double* pre,
                                double* ff, const int64_t* plane_slot, int n_planes, double* planes, void* stream)
{
    if (!valid(p) || !ogrid || !rgrid || !zgrid || !rho || !source || !ff) return MMA_ERR_ARG;
    if (p->n_rho > (int64_t)kThreads * kMaxRhoPerThread) return MMA_ERR_TOO_LARGE;
    if ((n_planes > 0) != (plane_slot != nullptr && planes != nullptr)) return MMA_ERR_ARG;
    const size_t smem = sizeof(double2) * (size_t)p->n_r;
    if (smem > 220 * 1024) return MMA_ERR_TOO_LARGE;
    cudaFuncSetAttribute(plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    plain_kernel<<<(unsigned)p->n_omega, kThreads, smem, (cudaStream_t)stream>>>(
        *p, ogrid, rgrid, zgrid, rho, source, reinterpret_cast<const double2*>(pre), reinterpret_cast<double2*>(ff),
        n_planes > 0 ? plane_slot : nullptr, reinterpret_cast<double2*>(planes));
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

extern "C" int mma_hankel_fast_plan(const double* zg, int64_t nz, double distance, double omega_max, double r_max,
                                    double rho_max, double tol, mma_hankel_fast_plan_t* plan)
{
    if (!zg || nz < 1 || !plan || !(tol > 0.0)) return MMA_ERR_ARG;
    double dmin = 1e300, dmax = -1e300;
    for (int64_t k = 0; k < nz; k++) {
        const double D = distance - zg[k];
        if (!(D > 0.0)) return MMA_ERR_ARG;
        dmin = D < dmin ? D : dmin;
        dmax = D > dmax ? D : dmax;
    }
    const double d_ref = std::sqrt(2.0 / (1.0 / (dmin * dmin) + 1.0 / (dmax * dmax)));
    double sigma = 0.0;
    for (int64_t k = 0; k < nz; k++) {
        const double l = d_ref / (distance - zg[k]);
        sigma = std::fabs(1.0 - l * l) > sigma ? std::fabs(1.0 - l * l) : sigma;
    }
    if (!(sigma > 1e-300)) sigma = 1.0;  // one distance only: v_k = 0, the m = 0 term is exact
    const double y_max = std::fabs(omega_max) / kC * std::fabs(r_max) * std::fabs(rho_max) / d_ref;
    const double x = 0.5 * sigma * y_max;
    // smallest M with x^M / M! e^x < tol (|J_m| <= 1 bounds the dropped tail)
    int need = -1;
    double term = 1.0;
    for (int m = 1; m <= 64; m++) {
        term *= x / m;
        if (term * std::exp(x) < tol) {
            need = m;
            break;
        }
    }
    if (need < 0) return MMA_ERR_UNSUPPORTED;
    int M = -1;
    for (int c : kTerms)
        if (c >= need && c >= 2) {
            M = c;
            break;
        }
    if (M < 0) return MMA_ERR_UNSUPPORTED;
    double t = 1.0;
    for (int m = 1; m <= M; m++) t *= x / m;
    plan->d_ref = d_ref;
    plan->sigma = sigma;
    plan->n_terms = M;
    plan->y_max = y_max;
    plan->trunc_bound = t * std::exp(x);
    return MMA_OK;
}

// scratch: B [n_omega][n_terms][n_r] complex float | per-plane table (n_z rows of n_terms + 4 floats)
// | ktab [n_omega] float2 | rtab [n_r] float4 | status word
static size_t up256(size_t v) { return (v + 255) / 256 * 256; }
static size_t bp_bytes(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return up256(sizeof(float2) * (size_t)p->n_omega * (size_t)plan->n_terms * (size_t)p->n_r);
}
static size_t ptab_bytes(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return up256(sizeof(float) * (size_t)p->n_z * (size_t)(plan->n_terms + 4));
}
static size_t ktab_off(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return bp_bytes(p, plan) + ptab_bytes(p, plan);
}
static size_t rtab_off(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return ktab_off(p, plan) + up256(sizeof(float2) * (size_t)p->n_omega);
}
static size_t status_off(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return rtab_off(p, plan) + up256(sizeof(float4) * (size_t)p->n_r);
}

// after the status word: the series planes' tables (sel_kz, vsel) and A_k rows (asel)
static size_t sel_off(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return status_off(p, plan) + 256;
}
static size_t asel_off(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    return sel_off(p, plan) + up256(64 + sizeof(float2) * (size_t)plan->n_terms);
}

extern "C" size_t mma_hankel_fast_scratch_bytes(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    if (!p || !plan) return 0;
    return asel_off(p, plan) + up256(sizeof(float2) * 2 * (size_t)p->n_omega * (size_t)p->n_r);
}

// The series cut-off of m terms for a plan (host only): the largest x = sigma y / 2 at which m
// terms meet the plan's truncation bound, -1 if m < 2.
extern "C" double mma_hankel_series_cut(const mma_hankel_fast_plan_t* plan, int m)
{
    return plan ? (double)series_cut(plan, m) : -1.0;
}

extern "C" int mma_hankel_test_ring_timeout(int on)
{
    g_ring_no_issue = on ? 1 : 0;
    return MMA_OK;
}

extern "C" int mma_hankel_set_stage1(int mode)
{
    if (mode != 0 && mode != 1) return MMA_ERR_ARG;
    g_stage1_mode = mode;
    return MMA_OK;
}

extern "C" int mma_hankel_fast_status(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan,
                                      const void* scratch, void* stream)
{
    if (!p || !plan || !scratch) return MMA_ERR_ARG;
    int h = 0;
    if (cudaMemcpyAsync(&h, static_cast<const char*>(scratch) + status_off(p, plan), sizeof(int),
                        cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        return MMA_ERR_CUDA;
    return h == 0 ? MMA_OK : MMA_ERR_TIMEOUT;
}

namespace {
// Ring stages of stage 1 that fit next to its tables (0: the ring form does not apply here).
template <int MM>
int ring_stages(const mma_hankel_problem* p, const void* src)
{
    if (p->source_c128 || p->pre_radial || (p->n_r & 1) || (p->omega_stride & 1) || (p->plane_stride & 1) ||
        (reinterpret_cast<uintptr_t>(src) & 15) || (MM % 4) || MM > 16)
        return 0;
    // two CTAs per SM: at most ~110 KB of shared memory each
    const size_t stage = (size_t)kG * kRingR * 8 + 16;
    const size_t tables = (size_t)p->n_z * (MM * 4 + 16) + (size_t)MM * 8 * kRingR + 64;
    const size_t budget = 110 * 1024;
    if (tables + 4 * stage > budget) return 0;  // at least four stages
    const size_t ns = (budget - tables) / stage;
    return (int)(ns > 16 ? 16 : ns);
}

template <int MM>
int launch_fast(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan, const double* og, const double* rg,
                const double* zg, const double* rho, const void* src, const double2* pre, double2* ff,
                float2* Bp, float* ptab, float2* ktab, float4* rtab, int* status, const int64_t* slot, int n_sel,
                double2* planes, int* sel_kz, float2* vsel, float2* asel, cudaStream_t st)
{
    const bool ser = n_sel > 0 && n_sel <= kSeriesPlanes;  // planes by the series inside stage 2
    fast_plane_table<MM><<<(unsigned)((p->n_z + 127) / 128), 128, 0, st>>>(*p, *plan, zg, ptab);
    bool ringed = false;
    if constexpr (MM % 4 == 0 && MM <= 16) {
        const int ns = ring_stages<MM>(p, src);
        int tc_done = 0;  // 1: stage 1 ran on the tensor cores
        if (ns > 0) {  // stage 1 through the shared-memory ring: on the tensor cores, or the CUDA cores
            ringed = true;
            const int64_t nt = p->n_omega > p->n_r ? p->n_omega : p->n_r;
            fast_wr_tables<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(*p, og, rg, ktab, rtab);
            if (g_stage1_mode == 0) {
                float uh, ul;
                const double u = 1.0 / (2.0 * plan->d_ref);
                uh = (float)u;
                ul = (float)(u - (double)uh);
                tc_done = mma::s1tc::stage1_tc_launch(*p, src, pre, ptab, ktab, rtab, make_float2(uh, ul), Bp, MM,
                                                      status, st);
                if (tc_done < 0) return tc_done;
            }
        }
        if (ns > 0 && tc_done == 0) {
            if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
            const size_t sr = (size_t)ns * kG * kRingR * 8 + (size_t)MM * 8 * kRingR +
                              (size_t)p->n_z * (MM * 4 + 16) + 2 * (size_t)ns * 8 + 16;
            float hi, lo;  // u_ref = 1/(2 d_ref) as a float pair
            const double u = 1.0 / (2.0 * plan->d_ref);
            hi = (float)u;
            lo = (float)(u - (double)hi);
            dim3 g1((unsigned)((p->n_r + kRingR - 1) / kRingR), (unsigned)p->n_omega);
            cudaFuncSetAttribute(fast_stage1_ring<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sr);
            fast_stage1_ring<MM><<<g1, kRingR + 32, sr, st>>>(*p, static_cast<const float2*>(src), pre, ptab, ktab,
                                                              rtab, make_float2(hi, lo), Bp, ns, status,
                                                              g_ring_no_issue);
        }
    }
    if (!ringed) {  // one thread per (frequency, radius) reading its planes directly
        const size_t s1 =
            sizeof(float) * (((size_t)p->n_z * (MM + 4) + 1) / 2 * 2) + sizeof(float2) * (size_t)p->n_z;
        if (s1 > 200 * 1024) return MMA_ERR_TOO_LARGE;
        cudaFuncSetAttribute(fast_stage1<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1);
        dim3 g1((unsigned)((p->n_r + kThreads - 1) / kThreads), (unsigned)p->n_omega);
        fast_stage1<MM><<<g1, kThreads, s1, st>>>(*p, og, rg, src, pre, ptab, Bp);
    }
    if (ser) {
        if (!ringed) {
            const int64_t nt = p->n_omega > p->n_r ? p->n_omega : p->n_r;
            fast_wr_tables<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(*p, og, rg, ktab, rtab);
        }
        series_plane_tables<<<1, 256, 0, st>>>(*p, *plan, zg, slot, n_sel, MM, sel_kz, vsel);
        dim3 ga((unsigned)((p->n_r + 255) / 256), (unsigned)p->n_omega, (unsigned)kSeriesPlanes);
        series_plane_a<MM><<<ga, 256, 0, st>>>(*p, ktab, rtab, ptab, src, pre, sel_kz, asel);
    }
    // stage 2: B, k r / d_ref and (series planes) their A_k rows per tile of rtile radii
    const int rows = MM + 1 + (ser ? kSeriesPlanes : 0);
    const size_t budget = (ser ? 72 : 96) * 1024;
    const size_t consts = (ser ? MM * (sizeof(float2) + 2 * sizeof(float4)) : MM * sizeof(float4));
    int rtile = (int)(p->n_r < 512 ? p->n_r : 512);
    rtile += rtile & 1;  // even row stride: stage 2 loads radius pairs as 16-byte words
    while ((size_t)rows * rtile * sizeof(float2) + consts > budget && rtile > 32) rtile /= 2;
    const size_t s2 = (size_t)rows * rtile * sizeof(float2) + consts;
    dim3 g2((unsigned)((p->n_rho + kThreads - 1) / kThreads), (unsigned)p->n_omega);
    const float cut8 = series_cut(plan, MM - 8), cut4 = series_cut(plan, MM - 4);
    if (ser) {
        cudaFuncSetAttribute(fast_stage2<MM, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
        fast_stage2<MM, true><<<g2, kThreads, s2, st>>>(*p, *plan, og, rg, rho, Bp, ff, rtile, asel, vsel, n_sel,
                                                         planes, cut8, cut4);
    } else {
        cudaFuncSetAttribute(fast_stage2<MM, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
        fast_stage2<MM, false><<<g2, kThreads, s2, st>>>(*p, *plan, og, rg, rho, Bp, ff, rtile, nullptr, nullptr, 0,
                                                          nullptr, cut8, cut4);
    }
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
}  // namespace

// FF[rho, w] = sum_k tau_k P_k[rho, w] (the z trapezoid) from plane transforms already computed:
// planes[slot[k]][rho][w], coalesced over w.  The kernel streams every plane once (HBM-bound).
// A CTA takes 64 elements; its four thread groups sum a quarter of the planes each (eight loads
// in flight per thread) and the quarters are added in a fixed order, so the result does not
// depend on scheduling.  Small work units keep the last wave of CTAs short (config 3: 8192 CTAs).
constexpr int kFfChunk = 512;  // planes whose offsets and weights are staged at a time
constexpr int kFfElems = 64;   // elements per CTA
__global__ void __launch_bounds__(kThreads) ff_from_planes_kernel(mma_hankel_problem P, const double* zg,
                                                                 const int64_t* slot, const double2* planes,
                                                                 double2* ff)
{
    constexpr int kGroups = kThreads / kFfElems;
    __shared__ int64_t s_off[kFfChunk];
    __shared__ double s_tau[kFfChunk];
    __shared__ double2 s_part[kGroups][kFfElems];
    const int64_t Nz = P.n_z, n = P.n_rho * P.n_omega;
    const int g = threadIdx.x / kFfElems;
    const int64_t e = blockIdx.x * (int64_t)kFfElems + threadIdx.x % kFfElems;
    const bool live = e < n;
    const int64_t a = live ? e : 0;  // clamped: every load stays in bounds
    double re = 0.0, im = 0.0;
    for (int64_t k0 = 0; k0 < Nz; k0 += kFfChunk) {
        const int nk = (int)(Nz - k0 < kFfChunk ? Nz - k0 : kFfChunk);
        __syncthreads();
        for (int q = threadIdx.x; q < nk; q += blockDim.x) {
            s_off[q] = slot[k0 + q] * n;
            s_tau[q] = trap_w(zg, k0 + q, Nz);
        }
        __syncthreads();
        const int per = (nk + kGroups - 1) / kGroups, q0 = g * per, q1 = q0 + per < nk ? q0 + per : nk;
        int q = q0;
        for (; q + 8 <= q1; q += 8) {
            double2 x[8];
#pragma unroll
            for (int u = 0; u < 8; u++) x[u] = __ldcs(planes + s_off[q + u] + a);
#pragma unroll
            for (int u = 0; u < 8; u++) {
                re = fma(s_tau[q + u], x[u].x, re);
                im = fma(s_tau[q + u], x[u].y, im);
            }
        }
        for (; q < q1; q++) {
            const double2 x = __ldcs(planes + s_off[q] + a);
            re = fma(s_tau[q], x.x, re);
            im = fma(s_tau[q], x.y, im);
        }
    }
    s_part[g][threadIdx.x % kFfElems] = make_double2(re, im);
    __syncthreads();
    if (g == 0 && live) {
        double2 acc = s_part[0][threadIdx.x];
#pragma unroll
        for (int q = 1; q < kGroups; q++) {
            acc.x += s_part[q][threadIdx.x].x;
            acc.y += s_part[q][threadIdx.x].y;
        }
        ff[e] = acc;
    }
}

extern "C" int mma_hankel_ff_from_planes(const mma_hankel_problem* p, const double* zgrid, const int64_t* plane_slot,
                                         const double* planes, double* ff, void* stream)
{
    if (!valid(p) || !zgrid || !plane_slot || !planes || !ff) return MMA_ERR_ARG;
    const int64_t n = p->n_rho * p->n_omega;
    const int64_t b = (n + kFfElems - 1) / kFfElems;
    if (b > INT32_MAX) return MMA_ERR_TOO_LARGE;
    ff_from_planes_kernel<<<(unsigned)b, kThreads, 0, (cudaStream_t)stream>>>(
        *p, zgrid, plane_slot, reinterpret_cast<const double2*>(planes), reinterpret_cast<double2*>(ff));
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

// A block of frequencies [n_z][w0:w1][n_r] copied between two sources laid out alike (host and
// device, either direction): n_z rows of block_bytes, the rows plane_bytes apart on both sides.
// One asynchronous 2-D copy on `stream`.
extern "C" int mma_hankel_copy_block(void* dst, const void* src, int64_t n_z, int64_t plane_bytes, int64_t block_bytes,
                                     void* stream)
{
    if (!dst || !src || n_z <= 0 || block_bytes <= 0 || plane_bytes < block_bytes) return MMA_ERR_ARG;
    return cudaMemcpy2DAsync(dst, (size_t)plane_bytes, src, (size_t)plane_bytes, (size_t)block_bytes, (size_t)n_z,
                             cudaMemcpyDefault, (cudaStream_t)stream) == cudaSuccess
               ? MMA_OK
               : MMA_ERR_CUDA;
}

extern "C" int mma_hankel_fast(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan, const double* ogrid,
                               const double* rgrid, const double* zgrid, const double* rho, const void* source,
                               const double* pre, double* ff, const int64_t* plane_slot, int n_planes,
                               double* planes, void* scratch, size_t scratch_bytes, void* stream)
{
    if (!valid(p) || !plan || !ogrid || !rgrid || !zgrid || !rho || !source || !ff) return MMA_ERR_ARG;
    if ((n_planes > 0) != (plane_slot != nullptr && planes != nullptr)) return MMA_ERR_ARG;
    if (!scratch || scratch_bytes < mma_hankel_fast_scratch_bytes(p, plan)) return MMA_ERR_ARG;
    if (!(plan->sigma > 0.0) || !(plan->d_ref > 0.0)) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const double2* pre2 = reinterpret_cast<const double2*>(pre);
    double2* ff2 = reinterpret_cast<double2*>(ff);
    char* sc = static_cast<char*>(scratch);
    float2* Bp = reinterpret_cast<float2*>(sc);
    float* ptab = reinterpret_cast<float*>(sc + bp_bytes(p, plan));
    float2* ktab = reinterpret_cast<float2*>(sc + ktab_off(p, plan));
    float4* rtab = reinterpret_cast<float4*>(sc + rtab_off(p, plan));
    int* status = reinterpret_cast<int*>(sc + status_off(p, plan));
    int* sel_kz = reinterpret_cast<int*>(sc + sel_off(p, plan));
    float2* vsel = reinterpret_cast<float2*>(sc + sel_off(p, plan) + 64);
    float2* asel = reinterpret_cast<float2*>(sc + asel_off(p, plan));
    double2* planes2 = reinterpret_cast<double2*>(planes);
    int rc;
#define MMA_FAST_CASE(T)                                                                                         \
    case T:                                                                                                      \
        rc = launch_fast<T>(p, plan, ogrid, rgrid, zgrid, rho, source, pre2, ff2, Bp, ptab, ktab, rtab, status,  \
                            plane_slot, n_planes, planes2, sel_kz, vsel, asel, st);                              \
        break;
    switch (plan->n_terms) {
        MMA_FAST_CASE(8)
        MMA_FAST_CASE(12)
        MMA_FAST_CASE(16)
        MMA_FAST_CASE(20)
        MMA_FAST_CASE(24)
        MMA_FAST_CASE(32)
        MMA_FAST_CASE(40)
        MMA_FAST_CASE(48)
        default: return MMA_ERR_ARG;
    }
#undef MMA_FAST_CASE
    if (rc != MMA_OK) return rc;
    if (n_planes > kSeriesPlanes) {  // more planes than the series pass takes: one J0 per term
        const int rtile = (int)(p->n_r < 1024 ? p->n_r : 1024);
        const size_t sp = 2 * sizeof(float2) * (size_t)rtile;
        dim3 gp((unsigned)((p->n_rho + kThreads - 1) / kThreads), (unsigned)p->n_omega, (unsigned)n_planes);
        fast_planes<<<gp, kThreads, sp, st>>>(*p, ogrid, rgrid, zgrid, rho, source, pre2, plane_slot,
                                              reinterpret_cast<double2*>(planes), rtile);
        if (cudaGetLastError() != cudaSuccess) return MMA_ERR_CUDA;
    }
    return MMA_OK;
}
