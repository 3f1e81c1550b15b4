/*
 * mma_diag.h -- measurement helpers of libmma_gb300.so (no counterpart in the reference).
 */
#ifndef MMA_DIAG_H
#define MMA_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

/* Peak fused-multiply-add rate of this GPU in FLOP/s (an FMA counts 2), measured
 * by a register-resident FMA loop over every SM: precision 0 = FP64, 1 = FP32.
 * Used as the roofline denominator of the arithmetic-bound kernels. */
int mma_probe_fma_peak(int precision, double *flops_per_s);

#ifdef __cplusplus
}
#endif
#endif
