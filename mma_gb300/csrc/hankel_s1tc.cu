// hankel_s1tc.cu -- the far field's stage 1 (the z contraction of the fast form) on the tensor
// cores: B_m[w, r] = sum_k tau_k v_k^m A_k[w, r] as, per frequency, a GEMM with rows (r, re/im),
// inner dimension the planes k and columns the series terms m, in TF32 split precision
// (hi*hi + hi*lo + lo*hi, FP32 accumulation in TMEM).
//
// One CTA per (frequency, 256 radii), 320 threads:
//   * warps 0-7 generate the A operand: thread g owns radius r0 + g and, per K-block of 8 planes,
//     forms A_k = pre_k S_k e^{-i delta_k} (the near-field phase relative to the per-radius
//     reference angle, as the CUDA-core ring form), splits Re and Im into TF32 hi + lo and stores
//     them as rows 2i, 2i+1 (i = g mod 64) of M-tile g / 64 (4 M-tiles of 128 rows);
//   * warp 8, lane 0 streams the source rows (one 1-D bulk copy per plane row) into a 4-stage
//     ring, 8 planes per stage;
//   * warp 9 allocates 64 TMEM columns (4 tiles x 16 terms) and its lane 0 issues, per K-block
//     and M-tile, three tcgen05.mma kind::tf32 (M 128, N 16, K 8) against the coefficient tile
//     C[m][k] = tau_k v_k^m (TF32 hi + lo, built once per CTA);
//   * warps 0-3 then read the accumulators (32x32b loads, one TMEM lane quadrant each), pair the
//     Re and Im rows by a shuffle, apply r w_r e^{-i k r^2 u_ref} and write B_m[w, r].
// Every mbarrier wait is bounded (time and a CTA-wide abort flag); on a timeout the CTA sets
// *status, drains its copies and MMAs, writes NaN into its B values and frees TMEM.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mma_hankel.h"
#include "../../include/mma_tdse.h"
#include "hankel_common.cuh"
#include "s1tc.cuh"
#include "tc_sm100.cuh"

namespace mma {
namespace s1tc {

using namespace tc;
using namespace hk;

constexpr uint64_t kSelfWaitNs = 20000000ull;  // 20 ms: the self-test's MMA completes in microseconds

// D[128][16] = A[128][8] B[16][8]^T by one tcgen05.mma kind::tf32 (M 128, N 16, K 8) from K-major
// core-matrix tiles (no swizzle: 16-byte K groups 128 bytes apart, 8-row groups 256 bytes apart).
// The wait for the MMA is bounded; on a timeout *status = 2 and D is not written.
__global__ void __launch_bounds__(128) s1tc_selftest_kernel(const float* A, const float* B, float* D, int* status)
{
    __shared__ __align__(1024) uint8_t sA[128 * 8 * 4];
    __shared__ __align__(1024) uint8_t sB[16 * 8 * 4];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int i = t; i < 128 * 8; i += 128)
        *reinterpret_cast<float*>(sA + plain_offset(i / 8, i % 8, 128, 256)) = A[i];
    for (int i = t; i < 16 * 8; i += 128)
        *reinterpret_cast<float*>(sB + plain_offset(i / 8, i % 8, 128, 256)) = B[i];
    if (t == 0) {
        mbar_init(&bar, 1);
        abort_s = 0;
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem_s, 32);
        tmem_relinquish();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_s;
    if (t == 0) {
        mma_tf32(tmem, sdesc_plain(smem_u32(sA), 128, 256), sdesc_plain(smem_u32(sB), 128, 256),
                 idesc_tf32_f32(128, 16), 0u);
        mma_commit(&bar);
    }
    __syncthreads();
    const bool ok = mbar_wait(&bar, 0u, &abort_s, kSelfWaitNs);
    if (!ok && lane == 0) atomicCAS(status, 0, 2);
    tc_fence_after();
    if (ok) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16), v);
#pragma unroll
        for (int c = 0; c < 16; c++) D[(warp * 32 + lane) * 16 + c] = v[c];
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

constexpr int kRows = 256;                        // radii per CTA
constexpr int kKB = 8;                            // planes per K-block (K of one TF32 MMA)
constexpr int kNSrc = 4;                          // source ring stages
constexpr int kNA = 2;                            // A-operand stages
constexpr int kTileBytes = 128 * kKB * 4;         // one M-tile of one K-block (hi or lo): 4 KB
constexpr int kAStage = 2 * 4 * kTileBytes;       // hi and lo of 4 M-tiles: 32 KB
constexpr int kSrcStage = kKB * kRows * 8;        // 16 KB
constexpr int kCTile = 16 * kKB * 4;              // 512 B per K-block (hi or lo)
constexpr uint64_t kWaitNs = 2000000000ull;       // 2 s per wait
constexpr uint32_t kLbo = 128, kSbo = 256;        // core-matrix strides of the tiles

__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void fail_s(volatile int* abort_s, int* status, int code)
{
    *abort_s = 1;
    atomicCAS(status, 0, code);
}

__global__ void __launch_bounds__(320, 1)
    stage1_tc_kernel(mma_hankel_problem P, const float2* __restrict__ src, const double2* __restrict__ pre,
                     const float* __restrict__ ptab, const float2* __restrict__ ktab, const float4* __restrict__ rtab,
                     float2 u_ref, float2* Bp, int* status)
{
    constexpr int MM = 16, RW = MM + 4;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float2* ring = reinterpret_cast<float2*>(sm);                     // kNSrc x kKB x kRows
    uint8_t* sA = sm + kNSrc * kSrcStage;                            // kNA x 32 KB
    uint8_t* sC = sA + kNA * kAStage;                                // nkb x (hi 512 B, lo 512 B)
    const int Nz = (int)P.n_z;
    const int nkb = (Nz + kKB - 1) / kKB;
    float4* pinfo = reinterpret_cast<float4*>(sC + (size_t)nkb * 2 * kCTile);  // Nz: (pre, du hi, du lo)
    uint64_t* bars = reinterpret_cast<uint64_t*>(pinfo + Nz);
    uint64_t *src_full = bars, *src_empty = bars + kNSrc, *a_full = bars + 2 * kNSrc,
             *a_empty = bars + 2 * kNSrc + kNA, *acc_full = bars + 2 * kNSrc + 2 * kNA, *drain = acc_full + 1;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_flag;
    __shared__ unsigned s_dumax;
    volatile int* abort_s = &abort_flag;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int64_t o = blockIdx.y, Nr = P.n_r, No = P.n_omega;
    const int64_t r0 = (int64_t)blockIdx.x * kRows;
    const int cnt = (int)(Nr - r0 < kRows ? Nr - r0 : kRows);
    const uint32_t row_bytes = (uint32_t)cnt * 8u;
    const float2* row0 = src + o * P.omega_stride + r0;
    if (t == 0) {
        for (int q = 0; q < kNSrc; q++) {
            mbar_init(&src_full[q], 1);
            mbar_init(&src_empty[q], 8);
        }
        for (int q = 0; q < kNA; q++) {
            mbar_init(&a_full[q], 8);
            mbar_init(&a_empty[q], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(drain, 1);
        abort_flag = 0;
        s_dumax = 0u;
        fence_barrier_init();
    }
    if (warp == 9) {
        tmem_alloc(&tmem_s, 64);
        tmem_relinquish();
    }
    // coefficient tiles C[m][k] = tau_k v_k^m (zero for padded planes) as TF32 hi + lo
    for (int q = t; q < nkb * kKB * MM; q += blockDim.x) {
        const int k = q / MM, m = q % MM;
        const float c = k < Nz ? ptab[k * RW + m] : 0.f;
        const float hi = tf32_rna(c), lo = tf32_rna(c - hi);
        uint8_t* base = sC + (size_t)(k / kKB) * 2 * kCTile;
        const uint32_t off = plain_offset(m, k % kKB, kLbo, kSbo);
        *reinterpret_cast<float*>(base + off) = hi;
        *reinterpret_cast<float*>(base + kCTile + off) = lo;
    }
    __syncthreads();  // barriers initialised, s_dumax zero
    {
        unsigned mx = 0u;
        for (int q = t; q < Nz; q += blockDim.x) {
            const double2 pf = pre ? pre[q * No + o] : make_double2(1.0, 0.0);
            const float duh = ptab[q * RW + MM + 2], dul = ptab[q * RW + MM + 3];
            pinfo[q] = make_float4((float)pf.x, (float)pf.y, duh, dul);
            mx = max(mx, __float_as_uint(fabsf(duh)));
        }
        atomicMax(&s_dumax, mx);
    }
    fence_async_smem();  // the coefficient tiles are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_s;
    // per-radius constants of the generator threads: k r^2 as float-float
    const int g = t;  // generator thread index (warps 0-7)
    const bool gen = warp < 8;
    const bool active = gen && g < cnt;
    const int64_t r = r0 + (active ? g : 0);
    const float2 kk = ktab[o];
    const float4 rt = rtab[r];
    const float kr2h = kk.x * rt.x;
    const float kr2l = fmaf(kk.x, rt.x, -kr2h) + fmaf(kk.x, rt.y, kk.y * rt.x);
    const bool near = P.near_field != 0;
    const bool small = __syncthreads_and(!active || fabsf(kr2h) * __uint_as_float(s_dumax) <= 0.12f);
    int n_issued_src = 0;
    bool mma_issued = false;
    if (gen) {
        // ------------------------------------------------------------ generators
        const int tq = g / 64, i = g % 64;
        const uint32_t row_re = 2 * i, row_im = 2 * i + 1;
        for (int j = 0; j < nkb && !*abort_s; j++) {
            const int ss = j % kNSrc, sa = j % kNA;
            if (!mbar_wait(&src_full[ss], (uint32_t)(j / kNSrc) & 1u, abort_s, kWaitNs)) {
                fail_s(abort_s, status, 1);
                break;
            }
            float2 a[kKB];
#pragma unroll
            for (int u = 0; u < kKB; u++) {
                const int k = j * kKB + u;
                a[u] = make_float2(0.f, 0.f);
                if (k < Nz && active) {
                    const float2 sv = ring[((size_t)ss * kKB + u) * kRows + g];
                    const float4 pf = pinfo[k];
                    float2 v = make_float2(fmaf(pf.x, sv.x, -pf.y * sv.y), fmaf(pf.x, sv.y, pf.y * sv.x));
                    if (near) {
                        float sn, cs;
                        if (small) {
                            sincos_small(kr2h * pf.z, sn, cs);
                        } else {
                            const float th = kr2h * pf.z;
                            const float te = fmaf(kr2h, pf.z, -th) + fmaf(kr2h, pf.w, kr2l * pf.z);
                            sincos_reduced(reduce_2pi(th, te), sn, cs);
                        }
                        v = make_float2(fmaf(v.x, cs, v.y * sn), fmaf(v.y, cs, -v.x * sn));
                    }
                    a[u] = v;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&src_empty[ss]);
            if (j >= kNA && !mbar_wait(&a_empty[sa], (uint32_t)((j - kNA) / kNA) & 1u, abort_s, kWaitNs)) {
                fail_s(abort_s, status, 2);
                break;
            }
            uint8_t* tile = sA + (size_t)sa * kAStage + (size_t)tq * kTileBytes;
#pragma unroll
            for (int h = 0; h < 2; h++) {  // K groups of 4 planes: one 16-byte chunk per row and part
                float4 rh, rl, ih, il;
                float* prh = &rh.x;
                float* prl = &rl.x;
                float* pih = &ih.x;
                float* pil = &il.x;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 v = a[4 * h + q];
                    prh[q] = tf32_rna(v.x);
                    prl[q] = tf32_rna(v.x - prh[q]);
                    pih[q] = tf32_rna(v.y);
                    pil[q] = tf32_rna(v.y - pih[q]);
                }
                *reinterpret_cast<float4*>(tile + plain_offset(row_re, 4 * h, kLbo, kSbo)) = rh;
                *reinterpret_cast<float4*>(tile + plain_offset(row_im, 4 * h, kLbo, kSbo)) = ih;
                *reinterpret_cast<float4*>(tile + 4 * kTileBytes + plain_offset(row_re, 4 * h, kLbo, kSbo)) = rl;
                *reinterpret_cast<float4*>(tile + 4 * kTileBytes + plain_offset(row_im, 4 * h, kLbo, kSbo)) = il;
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&a_full[sa]);
        }
    } else if (warp == 8) {
        // ------------------------------------------------------------ producer
        if (lane == 0)
            for (int j = 0; j < nkb && !*abort_s; j++) {
                const int ss = j % kNSrc;
                if (j >= kNSrc && !mbar_wait(&src_empty[ss], (uint32_t)((j - kNSrc) / kNSrc) & 1u, abort_s, kWaitNs)) {
                    fail_s(abort_s, status, 3);
                    break;
                }
                const int k0 = j * kKB, np = Nz - k0 < kKB ? Nz - k0 : kKB;
                mbar_arrive_expect_tx(&src_full[ss], row_bytes * (uint32_t)np);
                for (int u = 0; u < np; u++)
                    bulk_load_1d(ring + ((size_t)ss * kKB + u) * kRows, row0 + (int64_t)(k0 + u) * P.plane_stride,
                                 row_bytes, &src_full[ss]);
                n_issued_src = j + 1;
            }
    } else {
        // ------------------------------------------------------------ MMA issue
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32_f32(128, 16);
            for (int j = 0; j < nkb && !*abort_s; j++) {
                const int sa = j % kNA;
                if (!mbar_wait(&a_full[sa], (uint32_t)(j / kNA) & 1u, abort_s, kWaitNs)) {
                    fail_s(abort_s, status, 4);
                    break;
                }
                tc_fence_after();
                const uint32_t ab = smem_u32(sA + (size_t)sa * kAStage), cb = smem_u32(sC + (size_t)j * 2 * kCTile);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint32_t d = tmem + (uint32_t)(q * MM);
                    const uint64_t ahi = sdesc_plain(ab + q * kTileBytes, kLbo, kSbo);
                    const uint64_t alo = sdesc_plain(ab + (4 + q) * kTileBytes, kLbo, kSbo);
                    const uint64_t bhi = sdesc_plain(cb, kLbo, kSbo), blo = sdesc_plain(cb + kCTile, kLbo, kSbo);
                    mma_tf32(d, ahi, bhi, idesc, j > 0 ? 1u : 0u);
                    mma_tf32(d, ahi, blo, idesc, 1u);
                    mma_tf32(d, alo, bhi, idesc, 1u);
                }
                mma_issued = true;
                mma_commit(&a_empty[sa]);
            }
            if (!*abort_s) mma_commit(acc_full);
        }
    }
    __syncthreads();
    // after an abort: let the copies and MMAs already issued finish before the CTA leaves
    if (*abort_s) {
        if (warp == 8 && lane == 0)
            for (int j = (n_issued_src > kNSrc ? n_issued_src - kNSrc : 0); j < n_issued_src; j++)
                mbar_wait(&src_full[j % kNSrc], (uint32_t)(j / kNSrc) & 1u, nullptr, kWaitNs);
        if (warp == 9 && lane == 0 && mma_issued) {
            mma_commit(drain);
            mbar_wait(drain, 0u, nullptr, kWaitNs);
        }
    }
    __syncthreads();
    // ---------------------------------------------------------------- epilogue, warps 0-3
    if (warp < 4) {
        // warp-uniform: the TMEM loads below are warp-collective
        const bool ok = __all_sync(0xffffffffu, !*abort_s && mbar_wait(acc_full, 0u, abort_s, kWaitNs));
        tc_fence_after();
        const float nan = __int_as_float(0x7fc00000);
#pragma unroll 1
        for (int q = 0; q < 4; q++) {
            float v[16];
            if (ok) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(q * MM), v);
            const int rl = q * 64 + (warp * 32 + lane) / 2;  // this row pair's radius in the CTA
            const int64_t rr = r0 + rl;
            float2 bw = make_float2(0.f, 0.f);  // r w_r e^{-i k r^2 u_ref} of that radius
            if ((lane & 1) == 0 && rl < cnt) {
                const float4 rt2 = rtab[rr];
                const float h = kk.x * rt2.x;
                const float l = fmaf(kk.x, rt2.x, -h) + fmaf(kk.x, rt2.y, kk.y * rt2.x);
                bw = make_float2(rt2.z, 0.f);
                if (near) {
                    const float th = h * u_ref.x;
                    const float te = fmaf(h, u_ref.x, -th) + fmaf(h, u_ref.y, l * u_ref.x);
                    float sn, cs;
                    sincos_reduced(reduce_2pi(th, te), sn, cs);
                    bw = make_float2(rt2.z * cs, -rt2.z * sn);
                }
            }
#pragma unroll
            for (int m = 0; m < MM; m++) {
                const float mine = ok ? v[m] : 0.f;
                const float other = __shfl_xor_sync(0xffffffffu, mine, 1);
                if ((lane & 1) == 0 && rl < cnt) {
                    const float re = mine, im = other;
                    const float2 b = ok ? make_float2(fmaf(bw.x, re, -bw.y * im), fmaf(bw.x, im, bw.y * re))
                                        : make_float2(nan, nan);
                    Bp[(o * MM + m) * Nr + rr] = b;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 9) tmem_dealloc(tmem, 64);
}

}  // namespace s1tc
}  // namespace mma

// Tensor-core stage 1 (MM = 16 terms only), for complex64 sources whose plane rows start on 16-byte
// boundaries and pre-factors per (plane, frequency); returns 1 when it applies and was launched,
// 0 when the problem needs the CUDA-core stage 1, or an MMA_ERR_* status.
int mma::s1tc::stage1_tc_launch(const mma_hankel_problem& P, const void* src, const double2* pre, const float* ptab,
                                const float2* ktab, const float4* rtab, float2 u_ref, float2* Bp, int n_terms,
                                int* status, cudaStream_t st)
{
    if (n_terms != 16 || P.source_c128 || P.pre_radial || (P.n_r & 1) || (P.omega_stride & 1) ||
        (P.plane_stride & 1) || (reinterpret_cast<uintptr_t>(src) & 15) || P.n_omega > 65535)
        return 0;
    const int nkb = (int)((P.n_z + kKB - 1) / kKB);
    const size_t smem = 1024 + (size_t)kNSrc * kSrcStage + (size_t)kNA * kAStage + (size_t)nkb * 2 * kCTile +
                        (size_t)P.n_z * 16 + 16 * 8;
    if (smem > 227 * 1024) return 0;
    if (cudaFuncSetAttribute(stage1_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return MMA_ERR_CUDA;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    dim3 grid((unsigned)((P.n_r + kRows - 1) / kRows), (unsigned)P.n_omega);
    stage1_tc_kernel<<<grid, 320, smem, st>>>(P, static_cast<const float2*>(src), pre, ptab, ktab, rtab, u_ref, Bp,
                                             status);
    return cudaGetLastError() == cudaSuccess ? 1 : MMA_ERR_CUDA;
}

// Self-test of the TF32 tile layout (A [128][8], B [16][8] row-major FP32 in device memory,
// D [128][16]); *status becomes 2 if the bounded wait for the MMA ran out.
extern "C" int mma_s1tc_selftest(const float* A, const float* B, float* D, int* status, void* stream)
{
    if (!A || !B || !D || !status) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    mma::s1tc::s1tc_selftest_kernel<<<1, 128, 0, st>>>(A, B, D, status);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
