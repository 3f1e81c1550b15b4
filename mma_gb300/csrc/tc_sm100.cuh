// tc_sm100.cuh -- inline-PTX building blocks for 5th-generation tensor cores (sm_100 family):
// mbarriers with bounded waits, TMA tiled loads, TMEM allocation, tcgen05.mma (kind::f16,
// FP32 accumulation in TMEM), tcgen05.commit and tcgen05.ld.
//
// Shared-memory operand layout used throughout: K-major, 64-byte swizzle ("SW64"), the layout a
// TMA tiled load with CU_TENSOR_MAP_SWIZZLE_64B writes for a box whose inner extent is 32 FP16
// (64 bytes): row n of the tile occupies bytes [64 n, 64 n + 64), and within each 512-byte group
// of 8 rows the 16-byte chunk c of row n is stored at chunk position c ^ ((n >> 1) & 3).
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mma {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------------------------------ mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait until the phase with the given parity has completed.  Bounded: gives up after
// `limit_ns` nanoseconds, or as soon as *abort (a flag in shared memory; nullptr: bounded by
// time only) is set, and then returns false.  The caller records the failure and leaves its loop.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile int* abort,
                                          uint64_t limit_ns)
{
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 1;; i++) {
        if (mbar_test(bar, parity)) return true;
        if ((i & 63) == 0) {
            if (abort && *abort) return false;
            if (global_ns() - t0 > limit_ns) return false;
        }
    }
}

// 1-D bulk copy global -> shared (no tensor map) completing on an mbarrier's transaction count;
// both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// mbar_wait for waits that are usually short and frequent (once per ring stage per thread): up to
// 64 tests before the first read of the global timer
__device__ __forceinline__ bool mbar_wait_spin(uint64_t* bar, uint32_t parity, const volatile int* abort,
                                               uint64_t limit_ns)
{
#pragma unroll 1
    for (int i = 0; i < 64; i++)
        if (mbar_test(bar, parity)) return true;
    return mbar_wait(bar, parity, abort, limit_ns);
}

// L1 prefetch hint for an address inside an allocation
__device__ __forceinline__ void prefetch_l1(const void* p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// ------------------------------------------------------------------------ proxies and fences
// generic-proxy shared-memory writes become visible to the async proxy (tcgen05.mma, TMA)
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ------------------------------------------------------------------------ TMA
__device__ __forceinline__ void tma_prefetch(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// ------------------------------------------------------------------------ TMEM
// whole warp; the allocated base address is written to *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 lanes x 32 bits, 16 consecutive columns: thread t of the warp receives lane (base lane + t)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 32 bits, 32 consecutive columns (one load, one wait)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------------ MMA
// Instruction descriptor, kind::f16: FP16 A and B (both K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N)
{
    return (1u << 4)                          // D format: F32
           | (0u << 7) | (0u << 10)           // A, B format: F16
           | ((uint32_t)(N >> 3) << 17)       // N / 8
           | ((uint32_t)(M >> 4) << 24);      // M / 16
}

// Shared-memory matrix descriptor, K-major SW64: rows of 64 bytes, 8-row groups 512 bytes apart.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)  // start address / 16
           | ((uint64_t)1u << 16)                // leading byte offset (unused for swizzled K-major)
           | ((uint64_t)(512u >> 4) << 32)       // stride byte offset: 8 rows x 64 B
           | ((uint64_t)1u << 46)                // descriptor version (tcgen05)
           | ((uint64_t)4u << 61);               // layout: 64-byte swizzle
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// Instruction descriptor, kind::tf32: TF32 A and B (both K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32_f32(int M, int N)
{
    return (1u << 4)                          // D format: F32
           | (2u << 7) | (2u << 10)           // A, B format: TF32
           | ((uint32_t)(N >> 3) << 17)       // N / 8
           | ((uint32_t)(M >> 4) << 24);      // M / 16
}

// Shared-memory matrix descriptor, K-major without swizzle: core matrices of 8 rows x 16 bytes
// (128 contiguous bytes), `lbo` bytes between core matrices adjacent in K, `sbo` bytes between
// core matrices adjacent in M (or N).
__device__ __forceinline__ uint64_t sdesc_plain(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)   // start address / 16
           | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16)
           | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32)
           | ((uint64_t)1u << 46);               // descriptor version (tcgen05); layout: no swizzle
}

// byte offset of element (row, k) of a K-major TF32 tile stored as core matrices: 8-row groups
// `sbo` bytes apart, 4-element (16-byte) K groups `lbo` bytes apart
__host__ __device__ constexpr uint32_t plain_offset(uint32_t row, uint32_t k, uint32_t lbo, uint32_t sbo)
{
    return (row >> 3) * sbo + (k >> 2) * lbo + (row & 7u) * 16u + (k & 3u) * 4u;
}

// D[tmem] (+)= A[smem] * B[smem]^T with TF32 operands (K = 8 per instruction), issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// the mbarrier receives one arrival when all tcgen05.mma issued so far by this thread completed
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// byte offset of element (row, k) (k < 32, FP16) in a K-major SW64 tile
__device__ __forceinline__ uint32_t sw64_offset(uint32_t row, uint32_t k)
{
    return (row >> 3) * 512u + (row & 7u) * 64u + ((((k >> 3) ^ (row >> 1)) & 3u) << 4) + (k & 7u) * 2u;
}

}  // namespace tc
}  // namespace mma
