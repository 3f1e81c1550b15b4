// hankel_tc.cu -- per-plane far-field transforms of many planes on the 5th-generation tensor
// cores: the split-precision (three-term FP16, FP32 accumulation) form of
// Hankel/Hankel_transform.py:452-519 as called for every plane by Hankel_long (:523-686) when
// the cumulative results are requested.
//
// For frequency w and plane k (D_k = distance - z_k, y = k_w r rho / d_ref, lambda_k = d_ref/D_k):
//   P_k[w, rho] = sum_r J0(lambda_k y) A_k[w, r]
//              = sum_m v_k^m (sigma y / 2)^m J_m(y) / m! ... = sum_m v_k^m C_m[rho, k],
//   C_m[rho, k] = sum_r K_m[rho, r] A_k[w, r],   K_m(y) = (sigma y/2)^m J_m(y)/m!,
// (the Bessel multiplication theorem; v_k = (1 - lambda_k^2)/sigma).  Per frequency this is a
// GEMM with rows (rho, m), inner dimension r and columns (plane, re/im):
//   * B (the per-plane source tables A_k[w, r], scaled per row to |.| <= 1 and split into FP16
//     hi + lo) is prepared once by prep_b and read by TMA (64-byte swizzle);
//   * A (the kernel K_m, scaled per m to |.| <= 1 and split into FP16 hi + lo) is generated in
//     shared memory by groups of CUDA-core warps, one half-warp per rho row (J0/J1 seeds, then
//     the recurrence in m), the groups taking K-blocks round robin;
//   * one thread issues tcgen05.mma (M = 128, N = 256, K = 16): hi*hi + hi*lo + lo*hi into one of
//     two FP32 accumulators in TMEM (256 columns each), alternating per tile;
//   * the epilogue reads TMEM, applies v_k^m / s_m, reduces over m across lanes and writes the
//     requested planes (complex128, [slot][rho][w]).  The generator warps run it in chunks
//     between the next tile's K-blocks, so one accumulator drains while the tensor cores fill
//     the other.
// Every mbarrier wait is bounded (time and a CTA-wide abort flag); a timeout sets a status word
// and the kernel drains its tensor-core work and frees TMEM before returning.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <type_traits>

#include "../../include/mma_diag.h"
#include "../../include/mma_hankel.h"
#include "../../include/mma_tdse.h"
#include "hankel_common.cuh"
#include "tc_sm100.cuh"

namespace mma {
namespace hk {
namespace tcf {

using namespace mma::tc;

// packed FP32x2 helpers: a negated pair, a broadcast scalar
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }

constexpr int KB = 32;       // r per K-block: 32 FP16 = one 64-byte swizzled row
constexpr int NP = 128;      // planes per tile
constexpr int NCOL = 2 * NP; // accumulator columns of a tile (re, im per plane)
constexpr int NACC = 2;      // accumulators in TMEM (2 x 256 columns): tile n+1's MMAs run while tile n drains
constexpr int STAGES = 4;
constexpr int NGEN = 16;     // generator warps; they also run the epilogue
constexpr int THREADS = 32 * (2 + NGEN);
constexpr uint32_t A_BYTES = 128 * KB * 2;  // hi or lo: 8 KB
constexpr uint32_t B_BYTES = NCOL * KB * 2; // hi or lo: 16 KB
constexpr uint32_t B_OFF = 2 * A_BYTES;
constexpr uint32_t STAGE_BYTES = B_OFF + 2 * B_BYTES;  // 48 KB
constexpr uint64_t WAIT_NS = 2000000000ull;             // 2 s per wait
constexpr uint64_t kPrepWaitNs = 2000000000ull;         // 2 s per ring wait of the B preparation

struct Params {
    int64_t n_omega, n_r, n_z, n_rho;
    int64_t rpad, zpad;       // r padded to KB, planes padded to NP
    int64_t n_tiles, n_pb, n_rb;
    double inv_cd;            // 1 / (c d_ref): y = w r rho inv_cd
    float sigma;
    const double* og;
    const double* rg;
    const double* rho;
    const float* alpha;       // [n_omega][zpad]: scale of B rows (both re and im of plane k)
    const float* ftab;        // [zpad][MM]: v_k^m / s_m, plane-major
    const int64_t* slot;      // [n_z]
    double* planes;           // [n_planes][n_rho][n_omega] complex128
    int* status;
    const float2* rgf;        // [rpad] r as float-float (0 beyond n_r)
    const float2* krho;       // [n_omega][n_rho] w rho / (c d_ref) as float-float
    float inv_ymax, two_over_ymax;
    // y at or below which MM - 8 (MM - 4) series terms meet the plan's truncation bound: a K-block
    // whose largest y is below stores the higher terms of its A operand as zeros
    float ycut8, ycut4;
};

__device__ __forceinline__ void fail(volatile int* abort_s, int* status, int code)
{
    *abort_s = 1;
    atomicCAS(status, 0, code);
}

// reduce-scatter over G lanes of CH values: afterwards lane g of each group holds the group sum
// of columns (g % G) * (CH / G) + j, j < CH / G, in v[j]
template <int G, int CH>
__device__ __forceinline__ void reduce_scatter(float (&v)[CH], int lane)
{
    int n = CH;
#pragma unroll
    for (int d = G / 2; d >= 1; d >>= 1) {
        const bool up = (lane & d) != 0;
        const int h = n / 2;
#pragma unroll
        for (int i = 0; i < CH / 2; i++) {
            if (i < h) {
                const float send = up ? v[i] : v[i + h];
                const float keep = up ? v[i + h] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, send, d);
            }
        }
        n = h;
    }
}

template <int MM>
__global__ void __launch_bounds__(THREADS, 1)
    planes_tc_kernel(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo, Params P)
{
    constexpr int RC = 128 / MM;  // rho rows per tile (the 128 accumulator rows are (rho, m))
    constexpr int GW = RC / 2;    // warps of one generator group: a half-warp per rho row
    // groups, taking K-blocks round robin.  At most STAGES: a group's consecutive K-blocks are then
    // at most STAGES apart, so when it waits for a stage the stage's previous use has been waited
    // for (the parity wait cannot see a phase two behind); further warps only run the epilogue.
    constexpr int NG = NGEN / GW < STAGES ? NGEN / GW : STAGES;
    constexpr int CH = MM > 16 ? MM : 16;  // accumulator columns per reduction
    constexpr int CW = 32;                  // columns per TMEM load
    constexpr int EPI = NCOL / 4 / CW;      // epilogue chunks per warp: 4 warps share a lane quadrant
    static_assert(RC % 2 == 0 && NGEN % GW == 0, "generator groups");
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* full = bars;
    uint64_t* empty = bars + STAGES;
    uint64_t* acc_full = bars + 2 * STAGES;       // [NACC]
    uint64_t* acc_empty = acc_full + NACC;        // [NACC]
    uint64_t* drain = acc_empty + NACC;
    uint32_t* tmem_s = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_s = reinterpret_cast<volatile int*>(tmem_s + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nkb = (int)(P.rpad / KB);
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1 + GW);  // the producer + the generating group
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < NACC; a++) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], NGEN);
        }
        mbar_init(drain, 1);
        *abort_s = 0;
        fence_barrier_init();
    }
    if (warp == 1) {
        tmem_alloc(tmem_s, NACC * NCOL);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tma_prefetch(&tm_hi);
        tma_prefetch(&tm_lo);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_s;

    if (warp == 0) {
        // ---------------------------------------------------------------- TMA producer (B)
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; ok && tile < P.n_tiles; tile += gridDim.x) {
                const int64_t o = tile / (P.n_pb * P.n_rb), pb = (tile / P.n_rb) % P.n_pb;
                for (int kb = 0; kb < nkb; kb++, it++) {
                    const uint32_t s = it % STAGES, ph = (it / STAGES) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u, abort_s, WAIT_NS)) {
                        fail(abort_s, P.status, 1);
                        ok = false;
                        break;
                    }
                    uint8_t* st = smem + s * STAGE_BYTES + B_OFF;
                    mbar_arrive_expect_tx(&full[s], 2 * B_BYTES);
                    tma_load_3d(st, &tm_hi, &full[s], kb * KB, (int)(pb * NCOL), (int)o);
                    tma_load_3d(st + B_BYTES, &tm_lo, &full[s], kb * KB, (int)(pb * NCOL), (int)o);
                }
            }
            if (!ok) {  // let copies already issued land before the CTA leaves
                const uint64_t t0 = global_ns();
                while (global_ns() - t0 < 200000ull) {
                }
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16_f32(128, NCOL);
            uint32_t it = 0, tt = 0;
            bool ok = true;
            const uint32_t sbase = smem_u32(smem);
            for (int64_t tile = blockIdx.x; ok && tile < P.n_tiles; tile += gridDim.x, tt++) {
                const uint32_t a = tt % NACC;
                if (!mbar_wait(&acc_empty[a], ((tt / NACC) & 1u) ^ 1u, abort_s, WAIT_NS)) {
                    fail(abort_s, P.status, 2);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + a * (uint32_t)NCOL;
                for (int kb = 0; kb < nkb; kb++, it++) {
                    const uint32_t s = it % STAGES, ph = (it / STAGES) & 1u;
                    if (!mbar_wait(&full[s], ph, abort_s, WAIT_NS)) {
                        fail(abort_s, P.status, 3);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t st = sbase + s * STAGE_BYTES;
#pragma unroll
                    for (int ks = 0; ks < KB / 16; ks++) {
                        const uint64_t bh = sdesc_sw64(st + B_OFF + ks * 32);
                        const uint64_t bl = sdesc_sw64(st + B_OFF + B_BYTES + ks * 32);
                        const uint64_t ah = sdesc_sw64(st + ks * 32);
                        const uint64_t al = sdesc_sw64(st + A_BYTES + ks * 32);
                        mma_f16(d, ah, bh, idesc, (kb | ks) != 0);
                        mma_f16(d, ah, bl, idesc, 1u);
                        mma_f16(d, al, bh, idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&acc_full[a]);
            }
            // all MMAs this CTA issued complete before TMEM is freed -- also after an abort, so
            // this wait is bounded by time only, not by the abort flag
            mma_commit(drain);
            if (!mbar_wait(drain, 0u, nullptr, WAIT_NS)) fail(abort_s, P.status, 4);
        }
        __syncwarp();
    } else {
        // ---------------------------------------------------------------- generators + epilogue
        const int gw = warp - 2;
        const int grp = gw / GW, gwi = gw % GW;        // generator group (K-blocks it = grp mod NG), warp in it
        const int hw = lane >> 4, k0 = 2 * (lane & 15);  // half-warp -> rho row; lane -> r pair (k0, k0+1)
        const int q = 2 * gwi + hw;                      // this half-warp's rho row in the tile
        const int qd = warp % 4, cb = gw / 4;            // epilogue: TMEM lane quadrant, 64-column block
        const float tw = P.two_over_ymax, iy = P.inv_ymax;
        bool ok = true;
        // k rho / d_ref of this half-warp's row (float-float) for a tile, from the table
        auto row_of = [&](int64_t tile, float& kh, float& kl) {
            const int64_t o = tile / (P.n_pb * P.n_rb), rb = tile % P.n_rb;
            const int64_t ig = rb * RC + q;
            const float2 v = ig < P.n_rho ? __ldg(P.krho + o * P.n_rho + ig) : make_float2(0.f, 0.f);
            kh = v.x;
            kl = v.y;
        };
        // the A operand of K-block kb (this CTA's K-block number it) into its stage; false on timeout
        auto gen_block = [&](int kb, uint32_t it, float kh, float kl) -> bool {
            const uint32_t s = it % STAGES, ph = (it / STAGES) & 1u;
            // r and r+1 as float-float (hi0, lo0, hi1, lo1), loaded before the wait
            const float4 rv = __ldg(reinterpret_cast<const float4*>(P.rgf) + ((int64_t)kb * KB + k0) / 2);
            if (!mbar_wait(&empty[s], ph ^ 1u, abort_s, WAIT_NS)) {
                fail(abort_s, P.status, 5);
                return false;
            }
            // store addresses of this lane's pair (row q MM + m, columns k0, k0 + 1) in the SW64 layout:
            // q MM is a multiple of 8, so the 16-byte chunk is (k0 / 8) ^ ((m >> 1) & 3) and m enters
            // only through that class and a constant offset
            uint8_t* const base = smem + s * STAGE_BYTES + (q * MM / 8) * 512 + (k0 & 7) * 2;
            uint8_t* sa[4];
#pragma unroll
            for (int c = 0; c < 4; c++) sa[c] = base + ((((k0 >> 3) ^ c) & 3) << 4);
            // the lane's two radii as FP32x2 pairs: y = k rho r / d_ref in float-float
            const float2 rh = make_float2(rv.x, rv.z), rl = make_float2(rv.y, rv.w);
            const float2 yh = __fmul2_rn(bc2(kh), rh);
            const float2 yl = __fadd2_rn(__ffma2_rn(bc2(kh), rh, neg2(yh)), __ffma2_rn(bc2(kh), rl, __fmul2_rn(bc2(kl), rh)));
            float2 J0, J1;
            bessel01x2<true>(yh, yl, J0, J1);
            // K^_m = u^m J_m(y), u = y / y_max <= 1:  K^_{m+1} = (2m / y_max) K^_m - u^2 K^_{m-1}
            const float2 u = __fmul2_rn(__fadd2_rn(yh, yl), bc2(iy));
            const float2 w = __fmul2_rn(u, u);
            auto put2 = [&](int m, float2 x) {  // FP16 hi and lo of the pair
                const __half2 h = __float22half2_rn(x);
                const float2 f = __half22float2(h);
                const __half2 l = __float22half2_rn(__fadd2_rn(x, neg2(f)));
                uint8_t* const pa = sa[(m >> 1) & 3] + (m >> 3) * 512 + (m & 7) * 64;
                *reinterpret_cast<__half2*>(pa) = h;
                *reinterpret_cast<__half2*>(pa + A_BYTES) = l;
            };
            float2 a = J0, b = __fmul2_rn(u, J1);
            put2(0, a);
            put2(1, b);
            // terms up to ML - 1 by the recurrence, the rest zeros (ML warp-uniform)
            auto terms = [&](auto MLc) {
                constexpr int ML = decltype(MLc)::value;
#pragma unroll
                for (int m = 1; m + 1 < MM; m++) {
                    if (m + 1 < ML) {
                        const float2 n = __ffma2_rn(bc2((float)m * tw), b, neg2(__fmul2_rn(w, a)));
                        put2(m + 1, n);
                        a = b;
                        b = n;
                    } else {
                        uint8_t* const pa = sa[((m + 1) >> 1) & 3] + ((m + 1) >> 3) * 512 + ((m + 1) & 7) * 64;
                        *reinterpret_cast<uint32_t*>(pa) = 0u;
                        *reinterpret_cast<uint32_t*>(pa + A_BYTES) = 0u;
                    }
                }
            };
            const float ymx =
                __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(fmaxf(fabsf(yh.x), fabsf(yh.y)))));
            if (MM > 8 && ymx <= P.ycut8)
                terms(std::integral_constant<int, (MM > 8 ? MM - 8 : MM)>{});
            else if (MM > 4 && ymx <= P.ycut4)
                terms(std::integral_constant<int, (MM > 4 ? MM - 4 : MM)>{});
            else
                terms(std::integral_constant<int, MM>{});
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[s]);
            return true;
        };
        // chunk j (32 columns) of this warp's part of the epilogue of the tile in accumulator a:
        // TMEM -> v_k^m / s_m -> sum over m across lanes -> planes.  Chunk 0 waits for the tile's
        // MMAs; after the last one the warp releases the accumulator.
        auto epilogue = [&](int64_t tile, uint32_t tt, int j) -> bool {
            const uint32_t a = tt % NACC;
            const int64_t o = tile / (P.n_pb * P.n_rb), pb = (tile / P.n_rb) % P.n_pb, rb = tile % P.n_rb;
            if (j == 0) {
                {   // bring into L1 what this lane's epilogue reads: the per-plane factors of the 32
                    // planes of its column block and their slot and alpha entries
                    const int64_t kz0 = pb * NP + cb * (NCOL / 8);
                    for (int i = lane; i < (NCOL / 8) * MM / 32; i += 32) prefetch_l1(P.ftab + kz0 * MM + 32 * i);
                    if (lane < 2) prefetch_l1(P.slot + (kz0 + 16 * lane < P.n_z ? kz0 + 16 * lane : P.n_z - 1));
                    if (lane == 2) prefetch_l1(P.alpha + o * P.zpad + kz0);
                }
                if (!mbar_wait(&acc_full[a], (tt / NACC) & 1u, abort_s, WAIT_NS)) {
                    fail(abort_s, P.status, 6);
                    return false;
                }
                tc_fence_after();
            }
            const int row = qd * 32 + lane;
            const int m = row % MM;
            const float* fm = P.ftab + pb * NP * MM + m;
            const int64_t ig = rb * RC + row / MM;
            const int c0 = cb * (NCOL / 4) + j * CW;
            float f[CW / 2];  // factors of the 16 planes of these columns, requested first
#pragma unroll
            for (int i = 0; i < CW / 2; i++) f[i] = __ldg(fm + ((c0 >> 1) + i) * MM);
            float v[CW];
            tmem_ld32(tmem + ((uint32_t)(qd * 32) << 16) + a * (uint32_t)NCOL + (uint32_t)c0, v);
#pragma unroll
            for (int h = 0; h < CW / CH; h++) {
                float u[CH];
#pragma unroll
                for (int i = 0; i < CH; i++) u[i] = v[h * CH + i] * f[(h * CH + i) >> 1];
                reduce_scatter<MM, CH>(u, lane);
#pragma unroll
                for (int i = 0; i < CH / MM; i++) {
                    const int col = c0 + h * CH + (lane % MM) * (CH / MM) + i;
                    const int64_t kz = pb * NP + (col >> 1);
                    if (kz < P.n_z && ig < P.n_rho) {
                        const int64_t sl = __ldg(P.slot + kz);
                        if (sl >= 0)
                            P.planes[((sl * P.n_rho + ig) * P.n_omega + o) * 2 + (col & 1)] =
                                (double)(u[i] * __ldg(P.alpha + o * P.zpad + kz));
                    }
                }
            }
            if (j == EPI - 1) {
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[a]);
            }
            return true;
        };
        // Per tile: this group's K-blocks of the tile, each followed by one chunk of the previous
        // tile's epilogue (its accumulator drains while this tile's MMAs run on the other one);
        // the chunks left over (fewer K-blocks than chunks) and the last tile's epilogue after.
        uint32_t tt = 0;
        int64_t prev = -1;
        for (int64_t tile = blockIdx.x; ok && tile < P.n_tiles; tile += gridDim.x, tt++) {
            float kh, kl;
            row_of(tile, kh, kl);
            const uint32_t it0 = tt * (uint32_t)nkb;
            int j = 0;
            // this group's K-blocks: CTA-wide K-block numbers it = grp mod NG (not kb = grp mod NG,
            // which across a tile boundary would put up to 2 NG - 1 > STAGES blocks between two)
            const int kb0 = (int)((uint32_t)(grp + NG) - it0 % (uint32_t)NG) % NG;
            for (int kb = kb0; ok && grp < NG && kb < nkb; kb += NG) {
                ok = gen_block(kb, it0 + kb, kh, kl);
                if (ok && prev >= 0 && j < EPI) ok = epilogue(prev, tt - 1, j++);
            }
            for (; ok && prev >= 0 && j < EPI; j++) ok = epilogue(prev, tt - 1, j);
            prev = tile;
        }
        for (int j = 0; ok && prev >= 0 && j < EPI; j++) ok = epilogue(prev, tt - 1, j);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, NACC * NCOL);
    }
}

// k rho / d_ref per (frequency, screen radius) as float-float, for the A generators
__global__ void rho_table(const double* og, const double* rho, double inv_cd, int64_t n_omega, int64_t n_rho,
                          float2* krho)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_omega * n_rho) return;
    float h, l;
    split_d(og[i / n_rho] * inv_cd * rho[i % n_rho], h, l);
    krho[i] = make_float2(h, l);
}

// B operand: per (w, plane k) row the plane table A_k[w, r] = pre_k(w) e^{-i k r^2/(2 D_k)} r wr S_k[w, r]
// (FP32, float-float phase), scaled by 1/alpha (alpha = max over r of |Re|, |Im|) and split into
// FP16 hi + lo: Bh/Bl[w][2k + c][r], r padded to rpad, planes to zpad (zeros).
// One CTA per frequency; each thread owns r pairs.
constexpr int PREP_THREADS = 256;
constexpr int PREP_PAIRS = 2;  // rpad <= 2 * 2 * 256 = 1024

__global__ void __launch_bounds__(PREP_THREADS) prep_b(mma_hankel_problem P, float2 u_ref, const double* og,
                                                       const double* rg, const float4* dinv, const void* src,
                                                       const double2* pre,
                                                       __half* Bh, __half* Bl, float* alpha, int64_t rpad,
                                                       int64_t zpad)
{
    __shared__ float wmax[2][4][PREP_THREADS / 32];
    extern __shared__ float2 pre_s[];  // [zpad]: this frequency's pre-factor per plane, as floats
    const int64_t o = blockIdx.x, Nr = P.n_r, No = P.n_omega;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    // converted once per CTA: a double -> float conversion runs on the FP64 unit (a 32-lane
    // instruction holds a sub-partition's unit for about 64 cycles), so not per thread and plane
    for (int64_t kz = t; kz < zpad; kz += PREP_THREADS) {
        const double2 pf = (kz < P.n_z && pre && !P.pre_radial) ? pre[kz * No + o] : make_double2(1.0, 0.0);
        pre_s[kz] = make_float2((float)pf.x, (float)pf.y);
    }
    __syncthreads();
    float kh, kl;
    split_d(og[o] / kC, kh, kl);
    float kr2h[2 * PREP_PAIRS], kr2l[2 * PREP_PAIRS], wr[2 * PREP_PAIRS];
    float2 base[2 * PREP_PAIRS];  // e^{-i k r^2 u_ref} per radius (the near-field phase's reference part)
#pragma unroll
    for (int i = 0; i < 2 * PREP_PAIRS; i++) {
        const int64_t r = 2 * (t + (int64_t)PREP_THREADS * (i / 2)) + (i & 1);
        kr2h[i] = kr2l[i] = wr[i] = 0.f;
        base[i] = make_float2(1.f, 0.f);
        if (r < Nr) {
            const double rr = rg[r];
            float r2h, r2l;
            split_d(rr * rr, r2h, r2l);
            kr2h[i] = kh * r2h;
            kr2l[i] = fmaf(kh, r2h, -kr2h[i]) + fmaf(kh, r2l, kl * r2h);
            wr[i] = (float)(trap_w(rg, r, Nr) * rr);
            const float th = kr2h[i] * u_ref.x;
            const float te = fmaf(kr2h[i], u_ref.x, -th) + fmaf(kr2h[i], u_ref.y, kr2l[i] * u_ref.x);
            float sn, cs;
            sincos_reduced(reduce_2pi(th, te), sn, cs);
            base[i] = make_float2(cs, -sn);
        }
    }
    // the phase e^{-i k r^2 u_k} = base e^{-i delta}, delta = k r^2 (u_k - u_ref): by Taylor
    // polynomials when every |delta| of this CTA is within 0.12 (config 3: at most 0.033), else by
    // the exact float-float reduction; the choice is uniform over the CTA
    __shared__ unsigned s_dumax;
    if (t == 0) s_dumax = 0u;
    __syncthreads();
    {
        unsigned mx = 0u;
        for (int64_t kz = t; kz < P.n_z; kz += PREP_THREADS) mx = max(mx, __float_as_uint(fabsf(dinv[kz].z)));
        atomicMax(&s_dumax, mx);
    }
    __syncthreads();
    float kmax = 0.f;
#pragma unroll
    for (int i = 0; i < 2 * PREP_PAIRS; i++) kmax = fmaxf(kmax, fabsf(kr2h[i]));
    const bool small = __syncthreads_and(kmax * __uint_as_float(s_dumax) <= 0.12f);
    constexpr int PB = 4;  // planes per iteration: their loads are in flight together, one barrier for all
    for (int64_t kz0 = 0; kz0 < zpad; kz0 += PB) {
        float2 a[PB][2 * PREP_PAIRS];
        float mx[PB];
#pragma unroll
        for (int u = 0; u < PB; u++) {
            const int64_t kz = kz0 + u;
            const bool live = kz < P.n_z;
#pragma unroll
            for (int i = 0; i < 2 * PREP_PAIRS; i++) {
                const int64_t r = 2 * (t + (int64_t)PREP_THREADS * (i / 2)) + (i & 1);
                a[u][i] = (live && r < Nr) ? load_src_f(src, kz * P.plane_stride + o * P.omega_stride + r,
                                                        P.source_c128)
                                           : make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < PB; u++) {
            const int64_t kz = kz0 + u;
            const bool live = kz < P.n_z;
            const float2 pr0 = pre_s[kz];
            const float4 di = live ? dinv[kz] : make_float4(0.f, 0.f, 0.f, 0.f);
            mx[u] = 0.f;
#pragma unroll
            for (int i = 0; i < 2 * PREP_PAIRS; i++) {
                const float2 sv = a[u][i];
                float2 pr = pr0;
                if (P.pre_radial && live) {
                    const int64_t r = 2 * (t + (int64_t)PREP_THREADS * (i / 2)) + (i & 1);
                    if (r < Nr) {
                        const double2 pd = pre_at(P, pre, kz, o, r);
                        pr = make_float2((float)pd.x, (float)pd.y);
                    }
                }
                float2 v = make_float2(fmaf(pr.x, sv.x, -pr.y * sv.y), fmaf(pr.x, sv.y, pr.y * sv.x));
                if (P.near_field) {
                    float sn, cs;
                    if (small) {  // e^{-i theta} = base e^{-i delta}
                        sincos_small(kr2h[i] * di.z, sn, cs);
                        const float2 e = make_float2(fmaf(base[i].x, cs, base[i].y * sn),
                                                     fmaf(base[i].y, cs, -base[i].x * sn));
                        v = make_float2(fmaf(v.x, e.x, -v.y * e.y), fmaf(v.x, e.y, v.y * e.x));
                    } else {
                        const float th = kr2h[i] * di.x;
                        const float te = fmaf(kr2h[i], di.x, -th) + fmaf(kr2h[i], di.y, kr2l[i] * di.x);
                        sincos_reduced(reduce_2pi(th, te), sn, cs);  // e^{-i theta}
                        v = make_float2(fmaf(v.x, cs, v.y * sn), fmaf(v.y, cs, -v.x * sn));
                    }
                }
                a[u][i] = make_float2(v.x * wr[i], v.y * wr[i]);  // zero beyond n_r (wr = 0, source 0)
                mx[u] = fmaxf(mx[u], fmaxf(fabsf(a[u][i].x), fabsf(a[u][i].y)));
            }
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) mx[u] = fmaxf(mx[u], __shfl_xor_sync(0xffffffffu, mx[u], d));
        }
        const int par = (int)((kz0 / PB) & 1);
        if (lane == 0)
#pragma unroll
            for (int u = 0; u < PB; u++) wmax[par][u][w] = mx[u];
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PB; u++) {
            const int64_t kz = kz0 + u;
            float al = 0.f;
#pragma unroll
            for (int q = 0; q < PREP_THREADS / 32; q++) al = fmaxf(al, wmax[par][u][q]);
            const float sc = al > 0.f ? 1.0f / al : 0.f;
            if (t == 0) alpha[o * zpad + kz] = al;
#pragma unroll
            for (int pp = 0; pp < PREP_PAIRS; pp++) {
                const int64_t r0 = 2 * (t + (int64_t)PREP_THREADS * pp);
                if (r0 >= rpad) continue;
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const float x0 = (c ? a[u][2 * pp].y : a[u][2 * pp].x) * sc;
                    const float x1 = (c ? a[u][2 * pp + 1].y : a[u][2 * pp + 1].x) * sc;
                    const __half h0 = __float2half_rn(x0), h1 = __float2half_rn(x1);
                    const __half l0 = __float2half_rn(x0 - __half2float(h0)), l1 = __float2half_rn(x1 - __half2float(h1));
                    const int64_t idx = ((o * 2 * zpad + 2 * kz + c) * rpad + r0) / 2;
                    reinterpret_cast<__half2*>(Bh)[idx] = __halves2half2(h0, h1);
                    reinterpret_cast<__half2*>(Bl)[idx] = __halves2half2(l0, l1);
                }
            }
        }
    }
}

// The same B operand for complex64 sources whose plane rows start on 16-byte boundaries (an even
// number of radii at even strides) and pre-factors per (plane, frequency): thread 0 streams the
// frequency's rows into a shared-memory ring (one 1-D bulk copy per plane, kPrepG planes per
// stage, one mbarrier per stage), so the loads stay in flight across the per-stage barrier that
// the row scales need.  Each thread owns two radius pairs and carries every per-radius quantity
// as a pair, so the arithmetic runs in packed FP32x2 instructions: the same operations in the
// same order as prep_b, hence the same B operand bit for bit.  The wait for a stage is bounded;
// on a timeout the CTA sets *status, lets its copies land and writes NaN row scales.
constexpr int kPrepG = 4;  // planes per ring stage
__global__ void __launch_bounds__(PREP_THREADS, 2)
    prep_b_ring(mma_hankel_problem P, float2 u_ref, const double* og, const double* rg, const float4* dinv,
                const float2* __restrict__ src, const double2* __restrict__ pre, __half* Bh, __half* Bl,
                float* alpha, int64_t rpad, int64_t zpad, int ns, int* status)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(16) float wmax[2][kPrepG][PREP_THREADS / 32];  // double-buffered by stage parity
    __shared__ unsigned s_dumax;
    const int64_t o = blockIdx.x, Nr = P.n_r, No = P.n_omega;
    const int Nz = (int)P.n_z;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    float2* ring = reinterpret_cast<float2*>(smem_raw);                      // ns x kPrepG x rpad
    float4* pinfo = reinterpret_cast<float4*>(ring + (size_t)ns * kPrepG * rpad);  // zpad: (pre, du, 0)
    uint64_t* full = reinterpret_cast<uint64_t*>(pinfo + zpad);
    const int n_st = (int)((zpad + kPrepG - 1) / kPrepG);  // stages over the padded planes
    const int n_live = (Nz + kPrepG - 1) / kPrepG;         // stages with source rows to copy
    const uint32_t row_bytes = (uint32_t)Nr * 8u;
    const int rph = (int)(rpad / 2);  // half2 words per B row
    const float2* row0 = src + o * P.omega_stride;
    auto issue = [&](int j, int slot) {
        const int k0 = j * kPrepG, np = Nz - k0 < kPrepG ? Nz - k0 : kPrepG;
        tc::mbar_arrive_expect_tx(&full[slot], row_bytes * (uint32_t)np);
        for (int g = 0; g < np; g++)
            tc::bulk_load_1d(ring + ((size_t)slot * kPrepG + g) * rpad, row0 + (int64_t)(k0 + g) * P.plane_stride,
                             row_bytes, &full[slot]);
    };
    if (t == 0) {
        for (int q = 0; q < ns; q++) tc::mbar_init(&full[q], 1);
        s_dumax = 0u;
        tc::fence_barrier_init();
        for (int j = 0; j < n_live && j < ns; j++) issue(j, j);
    }
    __syncthreads();
    {
        unsigned mx = 0u;
        for (int64_t kz = t; kz < zpad; kz += PREP_THREADS) {
            const bool live = kz < Nz;
            const double2 pf = (live && pre) ? pre[kz * No + o] : make_double2(1.0, 0.0);
            const float du = live ? dinv[kz].z : 0.f;
            pinfo[kz] = make_float4((float)pf.x, (float)pf.y, du, 0.f);
            mx = max(mx, __float_as_uint(fabsf(du)));
        }
        atomicMax(&s_dumax, mx);
    }
    float kh, kl;
    split_d(og[o] / kC, kh, kl);
    // per radius pair (r0, r0 + 1), r0 = 2 (t + 256 pp): k r^2 as float-float, r w_r, and the
    // reference phase e^{-i k r^2 u_ref} = (bre, bim)
    float2 kr2h[PREP_PAIRS], kr2l[PREP_PAIRS], wr[PREP_PAIRS], bre[PREP_PAIRS], bim[PREP_PAIRS];
    float kmax = 0.f;
#pragma unroll
    for (int pp = 0; pp < PREP_PAIRS; pp++) {
        float v[5][2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int64_t r = 2 * (t + (int64_t)PREP_THREADS * pp) + q;
            v[0][q] = v[1][q] = v[2][q] = 0.f;
            v[3][q] = 1.f;
            v[4][q] = 0.f;
            if (r < Nr) {
                const double rr = rg[r];
                float r2h, r2l;
                split_d(rr * rr, r2h, r2l);
                v[0][q] = kh * r2h;
                v[1][q] = fmaf(kh, r2h, -v[0][q]) + fmaf(kh, r2l, kl * r2h);
                v[2][q] = (float)(trap_w(rg, r, Nr) * rr);
                const float th = v[0][q] * u_ref.x;
                const float te = fmaf(v[0][q], u_ref.x, -th) + fmaf(v[0][q], u_ref.y, v[1][q] * u_ref.x);
                float sn, cs;
                sincos_reduced(reduce_2pi(th, te), sn, cs);
                v[3][q] = cs;
                v[4][q] = -sn;
            }
            kmax = fmaxf(kmax, fabsf(v[0][q]));
        }
        kr2h[pp] = make_float2(v[0][0], v[0][1]);
        kr2l[pp] = make_float2(v[1][0], v[1][1]);
        wr[pp] = make_float2(v[2][0], v[2][1]);
        bre[pp] = make_float2(v[3][0], v[3][1]);
        bim[pp] = make_float2(v[4][0], v[4][1]);
    }
    __syncthreads();  // pinfo and s_dumax complete
    // the phase e^{-i k r^2 u_k} = base e^{-i delta}, delta = k r^2 (u_k - u_ref): Taylor polynomials
    // when every |delta| of this CTA is within 0.12, else the exact float-float reduction
    const bool small = __syncthreads_and(kmax * __uint_as_float(s_dumax) <= 0.12f);
    const bool near = P.near_field != 0;
    int s = 0;
    uint32_t ph = 0;
    int issued = n_live < ns ? n_live : ns;
    for (int j = 0; j < n_st; j++) {
        const int k0 = j * kPrepG;
        bool ok = true;
        if (j < n_live) ok = tc::mbar_wait_spin(&full[s], ph, nullptr, kPrepWaitNs);
        float2 are[kPrepG][PREP_PAIRS], aim[kPrepG][PREP_PAIRS];
        float mx[kPrepG];
#pragma unroll
        for (int u = 0; u < kPrepG; u++) {
            const int kz = k0 + u;
            const bool live = kz < Nz;
            const float4 pf = pinfo[kz < zpad ? kz : 0];
            const float2 prx = bc2(pf.x), pry = bc2(pf.y);
            mx[u] = 0.f;
#pragma unroll
            for (int pp = 0; pp < PREP_PAIRS; pp++) {
                const int64_t r0 = 2 * (t + (int64_t)PREP_THREADS * pp);
                float4 sv4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (live && r0 < Nr) sv4 = *reinterpret_cast<const float4*>(ring + ((size_t)s * kPrepG + u) * rpad + r0);
                const float2 sre = make_float2(sv4.x, sv4.z), sim = make_float2(sv4.y, sv4.w);
                // v = pre S
                float2 vre = __ffma2_rn(prx, sre, neg2(__fmul2_rn(pry, sim)));
                float2 vim = __ffma2_rn(prx, sim, __fmul2_rn(pry, sre));
                if (near) {
                    if (small) {  // e = base e^{-i delta}, then v e
                        const float2 d = __fmul2_rn(kr2h[pp], bc2(pf.z));
                        const float2 p2 = __fmul2_rn(d, d);
                        const float2 sn = __fmul2_rn(
                            d, __ffma2_rn(p2, __ffma2_rn(p2, bc2(8.33333333e-3f), bc2(-1.66666667e-1f)), bc2(1.0f)));
                        const float2 cs =
                            __ffma2_rn(p2, __ffma2_rn(p2, bc2(4.16666667e-2f), bc2(-0.5f)), bc2(1.0f));
                        const float2 ere = __ffma2_rn(bre[pp], cs, __fmul2_rn(bim[pp], sn));
                        const float2 eim = __ffma2_rn(bim[pp], cs, neg2(__fmul2_rn(bre[pp], sn)));
                        const float2 nre = __ffma2_rn(vre, ere, neg2(__fmul2_rn(vim, eim)));
                        const float2 nim = __ffma2_rn(vre, eim, __fmul2_rn(vim, ere));
                        vre = nre;
                        vim = nim;
                    } else {  // exact angle k r^2 / (2 D_k), per radius
                        const float4 di = live ? dinv[kz] : make_float4(0.f, 0.f, 0.f, 0.f);
                        float xr[2] = {vre.x, vre.y}, xi[2] = {vim.x, vim.y};
                        const float kh2[2] = {kr2h[pp].x, kr2h[pp].y}, kl2[2] = {kr2l[pp].x, kr2l[pp].y};
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            const float th = kh2[q] * di.x;
                            const float te = fmaf(kh2[q], di.x, -th) + fmaf(kh2[q], di.y, kl2[q] * di.x);
                            float sn, cs;
                            sincos_reduced(reduce_2pi(th, te), sn, cs);  // e^{-i theta}
                            const float a = fmaf(xr[q], cs, xi[q] * sn), b = fmaf(xi[q], cs, -xr[q] * sn);
                            xr[q] = a;
                            xi[q] = b;
                        }
                        vre = make_float2(xr[0], xr[1]);
                        vim = make_float2(xi[0], xi[1]);
                    }
                }
                are[u][pp] = __fmul2_rn(vre, wr[pp]);  // zero beyond n_r (wr = 0, source 0)
                aim[u][pp] = __fmul2_rn(vim, wr[pp]);
                mx[u] = fmaxf(mx[u], fmaxf(fmaxf(fabsf(are[u][pp].x), fabsf(aim[u][pp].x)),
                                           fmaxf(fabsf(are[u][pp].y), fabsf(aim[u][pp].y))));
            }
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) mx[u] = fmaxf(mx[u], __shfl_xor_sync(0xffffffffu, mx[u], d));
        }
        const int par = j & 1;
        if (lane == 0)
#pragma unroll
            for (int u = 0; u < kPrepG; u++) wmax[par][u][w] = mx[u];
        // every warp has read the stage (its slot can be refilled) and written its maxima
        if (__syncthreads_or(!ok)) {
            if (t == 0) {
                atomicCAS(status, 0, 1);
                for (int q = j; q < issued; q++)  // let the copies in flight land
                    tc::mbar_wait(&full[q % ns], (uint32_t)(q / ns) & 1u, nullptr, kPrepWaitNs);
            }
            for (int64_t kz = t; kz < zpad; kz += PREP_THREADS) alpha[o * zpad + kz] = __int_as_float(0x7fc00000);
            return;
        }
        if (t == 0 && issued < n_live) {
            issue(issued, s);  // stage j + ns into this stage's slot
            issued++;
        }
        if (j < n_live && ++s == ns) {
            s = 0;
            ph ^= 1u;
        }
        // the stage's rows start at row 2 k0 of this frequency; a row is rph half2 words and the
        // thread's pair pp sits at word t + 256 pp
        const int64_t row0 = (o * 2 * zpad + 2 * (int64_t)k0) * rph + t;
        __half2* bh = reinterpret_cast<__half2*>(Bh) + row0;
        __half2* bl = reinterpret_cast<__half2*>(Bl) + row0;
        const float4* wm = reinterpret_cast<const float4*>(&wmax[par][0][0]);
#pragma unroll
        for (int u = 0; u < kPrepG; u++) {
            if (k0 + u >= zpad) break;
            const float4 w0 = wm[2 * u], w1 = wm[2 * u + 1];  // the 8 warps' maxima
            const float al = fmaxf(fmaxf(fmaxf(w0.x, w0.y), fmaxf(w0.z, w0.w)), fmaxf(fmaxf(w1.x, w1.y), fmaxf(w1.z, w1.w)));
            const float sc = al > 0.f ? 1.0f / al : 0.f;
            if (t == 0) alpha[o * zpad + k0 + u] = al;
#pragma unroll
            for (int pp = 0; pp < PREP_PAIRS; pp++) {
                if (2 * (t + PREP_THREADS * pp) >= rpad) continue;
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const float2 x = __fmul2_rn(c ? aim[u][pp] : are[u][pp], bc2(sc));
                    const __half2 h = __float22half2_rn(x);
                    const float2 hb = __half22float2(h);
                    const __half2 l = __float22half2_rn(__fadd2_rn(x, neg2(hb)));
                    const int off = (2 * u + c) * rph + PREP_THREADS * pp;
                    bh[off] = h;
                    bl[off] = l;
                }
            }
        }
    }
}

// per plane: dinv = (1/(2 D_k) as (hi, lo), 1/(2 D_k) - 1/(2 d_ref), 0); ftab[k][m] = v_k^m / s_m =
// (v_k x)^m / m!, x = sigma y_max / 2;
// per radius: rgf = r as float-float
__global__ void plane_table(mma_hankel_problem P, mma_hankel_fast_plan_t F, const double* zg, const double* rg,
                            int mm, int64_t zpad, int64_t rpad, float4* dinv, float* ftab, float2* rgf)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < rpad; q += (int64_t)gridDim.x * blockDim.x) {
        float hi, lo;
        split_d(q < P.n_r ? rg[q] : 0.0, hi, lo);
        rgf[q] = make_float2(hi, lo);
    }
    const double x = 0.5 * F.sigma * F.y_max;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < zpad; q += (int64_t)gridDim.x * blockDim.x) {
        if (q >= P.n_z) {
            for (int m = 0; m < mm; m++) ftab[q * mm + m] = 0.f;
            continue;
        }
        const double D = P.distance - zg[q];
        const double lam = F.d_ref / D;
        const double v = (1.0 - lam * lam) / F.sigma;
        double c = 1.0;
        for (int m = 0; m < mm; m++) {
            ftab[q * mm + m] = (float)c;
            c *= (x > 0.0 ? v * x : v) / (double)(m + 1);
        }
        float hi, lo;
        split_d(1.0 / (2.0 * D), hi, lo);
        dinv[q] = make_float4(hi, lo, (float)(1.0 / (2.0 * D) - 1.0 / (2.0 * F.d_ref)), 0.f);
    }
}

// ------------------------------------------------------------------------ self-test
// One tile: D[128 x 256] = A[128 x 32] * B[256 x 32]^T in FP16 -> FP32, A staged by threads into
// the SW64 layout, B by threads (use_tma 0) or by TMA (1).  Checks descriptors, swizzle and the
// TMEM mapping.  use_tma 2 checks the bounded-wait path instead: thread 0 waits on a barrier that
// nothing arrives at (no copy, no MMA is issued), the wait runs out after kSelfTestWaitNs, the
// status word becomes 1 and the kernel frees its TMEM and returns without touching D.
constexpr uint64_t kSelfTestWaitNs = 20000000ull;
__global__ void __launch_bounds__(128) tc_selftest_kernel(const __grid_constant__ CUtensorMap tm_b, const __half* A,
                                                          const __half* B, float* D, int use_tma, int* status)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;
    uint8_t* sB = smem + 128 * 64;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + 256 * 64);
    uint32_t* tmem_s = reinterpret_cast<uint32_t*>(bars + 2);
    volatile int* abort_s = reinterpret_cast<volatile int*>(tmem_s + 1);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    for (int i = t; i < 128 * 32; i += 128)
        *reinterpret_cast<__half*>(sA + sw64_offset(i / 32, i % 32)) = A[i];
    if (!use_tma)
        for (int i = t; i < 256 * 32; i += 128)
            *reinterpret_cast<__half*>(sB + sw64_offset(i / 32, i % 32)) = B[i];
    if (t == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        *abort_s = 0;
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_s, 256);
        tmem_relinquish();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_s;
    bool ok = true;
    if (t == 0) {
        if (use_tma == 2) {  // nothing arrives at bars[0]: the bounded wait runs out
            if (!mbar_wait(&bars[0], 0u, abort_s, kSelfTestWaitNs)) {
                fail(abort_s, status, 1);
                ok = false;
            }
        } else if (use_tma) {
            mbar_arrive_expect_tx(&bars[0], 256 * 64);
            tma_load_3d(sB, &tm_b, &bars[0], 0, 0, 0);
            if (!mbar_wait(&bars[0], 0u, abort_s, WAIT_NS)) {
                fail(abort_s, status, 1);
                ok = false;
            }
        }
        if (ok) {
            constexpr uint32_t idesc = idesc_f16_f32(128, 256);
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
            for (int ks = 0; ks < 2; ks++) mma_f16(tmem, sdesc_sw64(a0 + ks * 32), sdesc_sw64(b0 + ks * 32), idesc, ks > 0);
            mma_commit(&bars[1]);
        }
    }
    __syncthreads();
    // after a failure nothing was committed to bars[1] (and the flag is set for every thread)
    if (!*abort_s && !mbar_wait(&bars[1], 0u, abort_s, WAIT_NS)) fail(abort_s, status, 2);
    tc_fence_after();
    if (!*abort_s) {
        for (int c0 = 0; c0 < 256; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; j++) D[(warp * 32 + lane) * 256 + c0 + j] = v[j];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

// ------------------------------------------------------------------------ host helpers
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder()
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// 3-D FP16 tensor [d2][d1][d0] (d0 contiguous), box {32, rows, 1}, 64-byte swizzle
bool make_map(CUtensorMap* map, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint32_t rows)
{
    EncodeTiled enc = encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {d0 * 2, d0 * d1 * 2};
    const cuuint32_t box[3] = {32, rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int tc_terms(int64_t n_terms)
{
    for (int c : {8, 16, 32})
        if (n_terms <= c) return c;
    return -1;
}

struct Layout {
    int mm;
    int64_t rpad, zpad;
    size_t off_bh, off_bl, off_alpha, off_ftab, off_dinv, off_rgf, off_krho, off_status, total;
};

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

bool layout(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan, Layout& L)
{
    L.mm = tc_terms(plan->n_terms);
    if (L.mm < 0) return false;
    L.rpad = (p->n_r + KB - 1) / KB * KB;
    L.zpad = (p->n_z + NP - 1) / NP * NP;
    if (L.rpad > 2 * 2 * PREP_THREADS) return false;
    if (sizeof(float2) * (size_t)L.zpad > 200 * 1024) return false;  // prep_b's per-plane table
    const size_t nb = (size_t)p->n_omega * 2 * L.zpad * L.rpad * sizeof(__half);
    L.off_bh = 0;
    L.off_bl = up256(nb);
    L.off_alpha = L.off_bl + up256(nb);
    L.off_ftab = L.off_alpha + up256(sizeof(float) * p->n_omega * L.zpad);
    L.off_dinv = L.off_ftab + up256(sizeof(float) * L.zpad * L.mm);
    L.off_rgf = L.off_dinv + up256(sizeof(float4) * L.zpad);
    L.off_krho = L.off_rgf + up256(sizeof(float2) * L.rpad);
    L.off_status = L.off_krho + up256(sizeof(float2) * p->n_omega * p->n_rho);
    L.total = L.off_status + 256;
    return true;
}

size_t planes_smem() { return 1024 + STAGES * STAGE_BYTES + 256; }  // alignment slack, stages, barriers

// Ring stages of the B preparation that fit two CTAs per SM (0: the ring form does not apply).
size_t prep_ring_smem(const Layout& L, int ns)
{
    return (size_t)ns * kPrepG * L.rpad * sizeof(float2) + (size_t)L.zpad * sizeof(float4) + (size_t)ns * 8;
}
int prep_ring_stages(const mma_hankel_problem* p, const void* src, const Layout& L)
{
    if (p->source_c128 || p->pre_radial || (p->n_r & 1) || (p->omega_stride & 1) || (p->plane_stride & 1) ||
        (reinterpret_cast<uintptr_t>(src) & 15))
        return 0;
    const size_t budget = 110 * 1024;
    const size_t stage = (size_t)kPrepG * L.rpad * sizeof(float2) + 8;
    const size_t fixed = (size_t)L.zpad * sizeof(float4);
    if (fixed + 2 * stage > budget) return 0;
    const size_t ns = (budget - fixed) / stage;
    return (int)(ns > 8 ? 8 : ns);
}

template <int MM>
int launch_planes(const CUtensorMap& th, const CUtensorMap& tl, const Params& P, cudaStream_t st)
{
    const size_t smem = planes_smem();
    if (cudaFuncSetAttribute(planes_tc_kernel<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return MMA_ERR_CUDA;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = P.n_tiles < sms ? P.n_tiles : sms;
    planes_tc_kernel<MM><<<(unsigned)grid, THREADS, smem, st>>>(th, tl, P);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

}  // namespace tcf
}  // namespace hk
}  // namespace mma

using namespace mma::hk;
using namespace mma::hk::tcf;

extern "C" size_t mma_hankel_planes_tc_scratch_bytes(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan)
{
    Layout L;
    if (!p || !plan || !layout(p, plan, L)) return 0;
    return L.total;
}

namespace {
// checks shared by the entry points; fills the scratch layout
int tc_check(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan, const double* ogrid, const double* rgrid,
             void* scratch, size_t scratch_bytes, Layout& L)
{
    if (!valid(p) || !plan || !ogrid || !rgrid) return MMA_ERR_ARG;
    if (!(plan->sigma > 0.0) || !(plan->d_ref > 0.0)) return MMA_ERR_ARG;
    if (!layout(p, plan, L)) return MMA_ERR_UNSUPPORTED;
    if (!scratch || scratch_bytes < L.total || (reinterpret_cast<uintptr_t>(scratch) & 255)) return MMA_ERR_ARG;
    if (p->n_omega > 2147483647LL || 2 * L.zpad > 2147483647LL) return MMA_ERR_TOO_LARGE;
    return MMA_OK;
}
}  // namespace

extern "C" int mma_hankel_planes_tc_prepare(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan,
                                            const double* ogrid, const double* rgrid, const double* zgrid,
                                            const void* source, const double* pre, void* scratch,
                                            size_t scratch_bytes, void* stream)
{
    Layout L;
    const int rc = tc_check(p, plan, ogrid, rgrid, scratch, scratch_bytes, L);
    if (rc != MMA_OK) return rc;
    if (!zgrid || !source) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* sc = static_cast<char*>(scratch);
    const int64_t nt = L.zpad > L.rpad ? L.zpad : L.rpad;
    plane_table<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(*p, *plan, zgrid, rgrid, L.mm, L.zpad, L.rpad,
                                                               reinterpret_cast<float4*>(sc + L.off_dinv),
                                                               reinterpret_cast<float*>(sc + L.off_ftab),
                                                               reinterpret_cast<float2*>(sc + L.off_rgf));
    float uh, ul;  // u_ref = 1/(2 d_ref) as a float pair
    {
        const double u = 1.0 / (2.0 * plan->d_ref);
        uh = (float)u;
        ul = (float)(u - (double)uh);
    }
    int* status = reinterpret_cast<int*>(sc + L.off_status) + 1;  // the preparation's own status word
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    const int ns = prep_ring_stages(p, source, L);
    if (ns > 0) {
        const size_t sr = prep_ring_smem(L, ns);
        if (cudaFuncSetAttribute(prep_b_ring, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sr) != cudaSuccess)
            return MMA_ERR_CUDA;
        prep_b_ring<<<(unsigned)p->n_omega, PREP_THREADS, sr, st>>>(
            *p, make_float2(uh, ul), ogrid, rgrid, reinterpret_cast<const float4*>(sc + L.off_dinv),
            static_cast<const float2*>(source), reinterpret_cast<const double2*>(pre),
            reinterpret_cast<__half*>(sc + L.off_bh), reinterpret_cast<__half*>(sc + L.off_bl),
            reinterpret_cast<float*>(sc + L.off_alpha), L.rpad, L.zpad, ns, status);
        return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
    }
    const size_t sp = sizeof(float2) * (size_t)L.zpad;
    if (sp > 48 * 1024 &&
        cudaFuncSetAttribute(prep_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp) != cudaSuccess)
        return MMA_ERR_CUDA;
    prep_b<<<(unsigned)p->n_omega, PREP_THREADS, sp, st>>>(
        *p, make_float2(uh, ul), ogrid, rgrid, reinterpret_cast<const float4*>(sc + L.off_dinv), source,
        reinterpret_cast<const double2*>(pre), reinterpret_cast<__half*>(sc + L.off_bh),
        reinterpret_cast<__half*>(sc + L.off_bl), reinterpret_cast<float*>(sc + L.off_alpha), L.rpad, L.zpad);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}

extern "C" int mma_hankel_planes_tc_run(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan,
                                        const double* ogrid, const double* rgrid, const double* rho,
                                        const int64_t* plane_slot, int n_planes, double* planes, void* scratch,
                                        size_t scratch_bytes, void* stream)
{
    Layout L;
    const int rc0 = tc_check(p, plan, ogrid, rgrid, scratch, scratch_bytes, L);
    if (rc0 != MMA_OK) return rc0;
    if (!rho || !plane_slot || !planes || n_planes < 1) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    char* sc = static_cast<char*>(scratch);
    int* status = reinterpret_cast<int*>(sc + L.off_status);
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    CUtensorMap th, tl;
    if (!make_map(&th, sc + L.off_bh, (uint64_t)L.rpad, (uint64_t)(2 * L.zpad), (uint64_t)p->n_omega, NCOL) ||
        !make_map(&tl, sc + L.off_bl, (uint64_t)L.rpad, (uint64_t)(2 * L.zpad), (uint64_t)p->n_omega, NCOL))
        return MMA_ERR_CUDA;
    Params P;
    std::memset(&P, 0, sizeof(P));
    P.n_omega = p->n_omega;
    P.n_r = p->n_r;
    P.n_z = p->n_z;
    P.n_rho = p->n_rho;
    P.rpad = L.rpad;
    P.zpad = L.zpad;
    const int rc = 128 / L.mm;  // rho rows per tile
    P.n_pb = L.zpad / NP;
    P.n_rb = (p->n_rho + rc - 1) / rc;
    P.n_tiles = p->n_omega * P.n_pb * P.n_rb;
    P.inv_cd = 1.0 / (kC * plan->d_ref);
    P.sigma = (float)plan->sigma;
    P.og = ogrid;
    P.rg = rgrid;
    P.rho = rho;
    P.alpha = reinterpret_cast<const float*>(sc + L.off_alpha);
    P.ftab = reinterpret_cast<const float*>(sc + L.off_ftab);
    P.slot = plane_slot;
    P.planes = planes;
    P.status = status;
    P.rgf = reinterpret_cast<const float2*>(sc + L.off_rgf);
    P.krho = reinterpret_cast<const float2*>(sc + L.off_krho);
    {
        const int64_t nk = p->n_omega * p->n_rho;
        rho_table<<<(unsigned)((nk + 255) / 256), 256, 0, st>>>(ogrid, rho, P.inv_cd, p->n_omega, p->n_rho,
                                                                 reinterpret_cast<float2*>(sc + L.off_krho));
        if (cudaGetLastError() != cudaSuccess) return MMA_ERR_CUDA;
    }
    P.inv_ymax = plan->y_max > 0.0 ? (float)(1.0 / plan->y_max) : 0.f;
    P.two_over_ymax = plan->y_max > 0.0 ? (float)(2.0 / plan->y_max) : 0.f;
    {   // x = sigma y / 2 cut-offs of the shorter series, as y (-1: never)
        const float x8 = series_cut(plan, L.mm - 8), x4 = series_cut(plan, L.mm - 4);
        P.ycut8 = x8 >= 0.f && plan->sigma > 0.0 ? (float)(2.0 * x8 / plan->sigma) : -1.f;
        P.ycut4 = x4 >= 0.f && plan->sigma > 0.0 ? (float)(2.0 * x4 / plan->sigma) : -1.f;
    }
    switch (L.mm) {
        case 8: return launch_planes<8>(th, tl, P, st);
        case 16: return launch_planes<16>(th, tl, P, st);
        case 32: return launch_planes<32>(th, tl, P, st);
        default: return MMA_ERR_UNSUPPORTED;
    }
}

extern "C" int mma_hankel_planes_tc(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan,
                                    const double* ogrid, const double* rgrid, const double* zgrid, const double* rho,
                                    const void* source, const double* pre, const int64_t* plane_slot, int n_planes,
                                    double* planes, void* scratch, size_t scratch_bytes, void* stream)
{
    const int rc = mma_hankel_planes_tc_prepare(p, plan, ogrid, rgrid, zgrid, source, pre, scratch, scratch_bytes,
                                                stream);
    if (rc != MMA_OK) return rc;
    return mma_hankel_planes_tc_run(p, plan, ogrid, rgrid, rho, plane_slot, n_planes, planes, scratch, scratch_bytes,
                                    stream);
}

extern "C" int mma_hankel_planes_tc_status(const mma_hankel_problem* p, const mma_hankel_fast_plan_t* plan,
                                           const void* scratch, void* stream)
{
    Layout L;
    if (!p || !plan || !scratch || !layout(p, plan, L)) return MMA_ERR_ARG;
    int h[2] = {0, 0};  // the tensor-core kernel's and the B preparation's status words
    if (cudaMemcpyAsync(h, static_cast<const char*>(scratch) + L.off_status, sizeof(h), cudaMemcpyDeviceToHost,
                        (cudaStream_t)stream) != cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        return MMA_ERR_CUDA;
    return (h[0] == 0 && h[1] == 0) ? MMA_OK : MMA_ERR_TIMEOUT;
}

extern "C" int mma_tc_selftest(const void* A, const void* B, float* D, int use_tma, int* status, void* stream)
{
    if (!A || !B || !D || !status) return MMA_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    CUtensorMap tb;
    std::memset(&tb, 0, sizeof(tb));
    if (use_tma < 0 || use_tma > 2) return MMA_ERR_ARG;
    if (use_tma == 1 && !make_map(&tb, B, 32, 256, 1, 256)) return MMA_ERR_CUDA;
    const size_t smem = 1024 + 128 * 64 + 256 * 64 + 64;
    if (cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return MMA_ERR_CUDA;
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return MMA_ERR_CUDA;
    tc_selftest_kernel<<<1, 128, smem, st>>>(tb, static_cast<const __half*>(A), static_cast<const __half*>(B), D,
                                              use_tma, status);
    return cudaGetLastError() == cudaSuccess ? MMA_OK : MMA_ERR_CUDA;
}
