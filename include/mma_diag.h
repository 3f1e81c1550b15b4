/*
 * mma_diag.h -- measurement helpers of libmma_gb300.so (no counterpart in the reference).
 */
#ifndef MMA_DIAG_H
#define MMA_DIAG_H

#include "mma_hankel.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Peak fused-multiply-add rate of this GPU in FLOP/s (an FMA counts 2), measured
 * by a register-resident FMA loop over every SM: precision 0 = FP64, 1 = FP32.
 * Used as the roofline denominator of the arithmetic-bound kernels. */
int mma_probe_fma_peak(int precision, double *flops_per_s);

/* Self-test of the tensor-core building blocks used by mma_hankel_planes_tc: one tile
 * D[128][256] = A[128][32] * B[256][32]^T with FP16 A, B (row-major, device pointers) and FP32 D,
 * through tcgen05.mma with the operands in 64-byte-swizzled shared memory.  A is staged by
 * threads; B by threads (use_tma = 0) or by a TMA tiled load (use_tma = 1).  *status (device)
 * is 0 on success, non-zero if a bounded wait gave up.
 * use_tma = 2 checks the failure path of those bounded waits: one thread waits on a barrier
 * that nothing arrives at (no copy and no MMA is issued), the wait gives up after 20 ms,
 * *status becomes 1, and the kernel frees its tensor memory and returns without writing D;
 * the context stays usable. */
int mma_tc_selftest(const void *A, const void *B, float *D, int use_tma, int *status, void *stream);
/* One tcgen05.mma kind::tf32 (M 128, N 16, K 8) from K-major core-matrix tiles without swizzle,
 * the operand layout of the tensor-core stage 1 of the fast far field: D[128][16] = A[128][8]
 * B[16][8]^T (row-major FP32, device pointers); *status = 2 if the bounded wait for the MMA ran out. */
int mma_s1tc_selftest(const float *A, const float *B, float *D, int *status, void *stream);

/* Test of the bounded waits of mma_hankel_fast's ring stage 1: while `on` is set, the ring's
 * copies are never issued, so every wait of the stage runs out after its 2 s limit; the call
 * returns, its far field is NaN and mma_hankel_fast_status reports MMA_ERR_TIMEOUT.  Process-wide;
 * for tests only. */
int mma_hankel_test_ring_timeout(int on);

/* The series cut-off behind the fast far field's choice of series length (host only, no device):
 * the largest x = sigma y / 2 at which m terms still meet plan->trunc_bound, x^m / m! e^x <=
 * trunc_bound; -1 for m < 2.  Stage 2 and the tensor-core generators take m = MM - 8 or MM - 4
 * terms where a chunk's largest y is within it. */
double mma_hankel_series_cut(const mma_hankel_fast_plan_t *plan, int m);

#ifdef __cplusplus
}
#endif
#endif
