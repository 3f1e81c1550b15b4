/*
 * mma_hankel.h -- C-ABI of the GB300 far-field (Hankel) kernels in libmma_gb300.so.
 *
 * Replaces the computational core of Hankel/Hankel_transform.py:
 *   HankelTransform (:452-519)  per-plane transform
 *       P_k[w, rho] = trapz_r( pre_k(w) e^{-i k r^2/(2 D_k)} r S_k[w, r] J0(k r rho / D_k) ),
 *       k = w/c, D_k = distance - z_k (the near-field factor optional)
 *   Hankel_long (:523-686)      z-trapezoid of the planes, entry/exit planes
 * Grids are SI; all pointers are device pointers; complex arrays are interleaved
 * (re, im).  Outputs use the reference's layout after its transposes: [rho][omega].
 */
#ifndef MMA_HANKEL_H
#define MMA_HANKEL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 8-byte fields only (same layout in every ABI). */
typedef struct mma_hankel_problem {
    int64_t n_omega, n_r, n_z, n_rho; /* n_z = planes used (the reference drops the last plane, :62) */
    double distance;                  /* screen distance from the first medium point (Hankel_long `distance`) */
    int64_t near_field;               /* 1 = apply e^{-i k r^2/(2 D_k)} (the reference default) */
    int64_t source_c128;              /* 0 = complex64 source, 1 = complex128 */
    int64_t plane_stride;             /* source elements between planes k */
    int64_t omega_stride;             /* source elements between frequencies; r is contiguous */
    int64_t pre_radial;               /* 0: pre [n_z][n_omega]; 1: pre [n_z][n_omega][n_r] (radially modulated
                                         medium, Hankel_transform.py:244-399, applied per radius as in :505-512) */
} mma_hankel_problem;

/* Inputs common to both forms:
 *   ogrid [n_omega], rgrid [n_r], zgrid [n_z], rho [n_rho]    float64 grids
 *   source                                                    S[k][w][r] with the strides above
 *   pre     [n_z][n_omega] complex128 pre-factor, or NULL for 1 (get_propagation_pre_factor_function);
 *           with pre_radial = 1, [n_z][n_omega][n_r]
 * Outputs:
 *   ff      [n_rho][n_omega] complex128                        FF_integrated
 *   plane_slot [n_z] int64 (or NULL): slot of plane k in `planes`, -1 = not stored;
 *           n_planes = number of slots in use (0..n_planes-1, each used once)
 *   planes  [n_planes][n_rho][n_omega] complex128 (or NULL)    per-plane transforms */

/* Plain form: the reference's arithmetic in FP64, one J0 (CUDA j0) per (w, k, rho, r)
 * term.  One CTA per frequency. */
int mma_hankel_plain(const mma_hankel_problem *p, const double *ogrid, const double *rgrid, const double *zgrid,
                     const double *rho, const void *source, const double *pre, double *ff,
                     const int64_t *plane_slot, int n_planes, double *planes, void *stream);

/* Parameters of the fast form, chosen on the host from the grids by mma_hankel_fast_plan. */
typedef struct mma_hankel_fast_plan_t {
    double d_ref;     /* reference distance: lambda_k = d_ref / D_k */
    double sigma;     /* max_k |1 - lambda_k^2| */
    int64_t n_terms;  /* terms of the multiplication-theorem series */
    double y_max;     /* largest k r rho / d_ref */
    double trunc_bound; /* bound on the truncation error relative to the largest |J0| term */
} mma_hankel_fast_plan_t;

/* Fast form (the chosen form): J0(lambda y) = sum_m ((1 - lambda^2) y / 2)^m / m! J_m(y)
 * (Bessel multiplication theorem) separates the plane distance from the (r, rho) kernel,
 * so the z-trapezoid is contracted first:
 *   B_m[w, r]   = sum_k tau_k v_k^m A_k[w, r],  v_k = (1 - lambda_k^2)/sigma     (HBM-bound)
 *   FF[rho, w]  = sum_{r, m} K_m(k r rho / d_ref) B_m[w, r],
 *   K_m(y) = (sigma y / 2)^m J_m(y) / m!, by a division-free recurrence from J0, J1. (FP32)
 * FP32 arithmetic, float-float phases, compensated sums.  Planes requested through plane_slot:
 * up to two (n_planes <= 2, e.g. the entry and exit planes) come from the same series in the
 * second stage, P_k[rho, w] = sum_r A_k[w, r] sum_m v_k^m K_m(y), sharing its K_m evaluations;
 * more are evaluated directly (FP32, one J0 per term).
 * The host fills `plan` with mma_hankel_fast_plan (zgrid on the host). */
int mma_hankel_fast_plan(const double *zgrid_host, int64_t n_z, double distance, double omega_max, double r_max,
                         double rho_max, double tol, mma_hankel_fast_plan_t *plan);
size_t mma_hankel_fast_scratch_bytes(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan);
/* FF[rho][w] = sum_k tau_k planes[plane_slot[k]][rho][w] (tau: trapezoid weights of zgrid), the
 * integrated far field from plane transforms already computed for every plane (plane_slot >= 0
 * for all n_z planes; complex128 planes [slot][n_rho][n_omega], ff [n_rho][n_omega]). */
int mma_hankel_ff_from_planes(const mma_hankel_problem *p, const double *zgrid, const int64_t *plane_slot,
                              const double *planes, double *ff, void *stream);
/* Stage 1 of mma_hankel_fast (the z contraction B_m): mode 1 (default) runs it on the CUDA cores
 * (FP32 FMAs, the streamed ring form); mode 0 runs it on the tensor cores where it applies -- 16
 * series terms, a complex64 source with rows on 16-byte boundaries (even n_r and strides),
 * pre-factors per (plane, frequency), at most about 1000 planes -- as a TF32 split-precision GEMM
 * (tcgen05, FP32 accumulation in TMEM).  On config 3 the tensor-core form is slower and less
 * accurate (per-harmonic error 6.6e-6 against 3.4e-7).  Process-wide setting; MMA_ERR_ARG for
 * other modes. */
int mma_hankel_set_stage1(int mode);
/* Status of the last mma_hankel_fast call on this scratch (synchronises the stream): MMA_OK, or
 * MMA_ERR_TIMEOUT if a bounded wait of its streamed stage 1 gave up (that call's far field is then
 * NaN).  The streamed stage 1 runs for complex64 sources with rows on 16-byte boundaries (even
 * n_r and strides) and pre-factors per (plane, frequency); other problems take the direct stage 1,
 * which has no waits. */
int mma_hankel_fast_status(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan, const void *scratch,
                           void *stream);
/* Copy of the frequency block [n_z][w0:w1][n_r] of a source between host and device (either
 * direction; the two sides laid out alike): n_z rows of block_bytes, plane_bytes apart on both
 * sides, as one asynchronous copy on `stream`.  The far field of a pinned host source uploads it
 * block by block with this and runs each block's fast form while the next block is in flight
 * (the fast form's per-frequency work is independent, so the result equals the one-shot call). */
int mma_hankel_copy_block(void *dst, const void *src, int64_t n_z, int64_t plane_bytes, int64_t block_bytes,
                          void *stream);
int mma_hankel_fast(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan, const double *ogrid,
                    const double *rgrid, const double *zgrid, const double *rho, const void *source, const double *pre,
                    double *ff, const int64_t *plane_slot, int n_planes, double *planes, void *scratch,
                    size_t scratch_bytes, void *stream);

/* Tensor-core form of the per-plane transforms (the split-precision form), for calls that
 * request many planes (the cumulative results of Hankel_long, :640-672).  Same series as
 * mma_hankel_fast with the number of terms rounded up to 8, 16 or 32, arranged per frequency as
 * a GEMM with rows (rho, m), inner dimension r, columns (plane, re/im):
 *   B = per-plane tables A_k[w, r] (FP16 hi + lo, scaled per row), read by TMA;
 *   A = K_m(k r rho / d_ref) scaled per m (FP16 hi + lo), generated on CUDA cores;
 *   tcgen05.mma hi*hi + hi*lo + lo*hi into FP32 accumulators in TMEM; the epilogue applies
 *   v_k^m and reduces over m.
 * Writes planes[plane_slot[k]] for every k with plane_slot[k] >= 0 (n_planes >= 1).
 * Requires n_r <= 1024 and a plan with n_terms <= 32 (else MMA_ERR_UNSUPPORTED).  Scratch of
 * mma_hankel_planes_tc_scratch_bytes (256-byte aligned).  mma_hankel_planes_tc_status
 * synchronises the stream and returns MMA_ERR_TIMEOUT if a bounded wait in the kernel gave up. */
size_t mma_hankel_planes_tc_scratch_bytes(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan);
int mma_hankel_planes_tc(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan, const double *ogrid,
                         const double *rgrid, const double *zgrid, const double *rho, const void *source,
                         const double *pre, const int64_t *plane_slot, int n_planes, double *planes, void *scratch,
                         size_t scratch_bytes, void *stream);
int mma_hankel_planes_tc_status(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan,
                                const void *scratch, void *stream);
/* The two halves of mma_hankel_planes_tc: _prepare builds the per-plane tables and the B operand
 * in scratch (depends on the source, pre-factor, grids and plan); _run launches the tensor-core
 * kernel (depends on rho, within the plan's y_max, and on the requested planes). */
int mma_hankel_planes_tc_prepare(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan,
                                 const double *ogrid, const double *rgrid, const double *zgrid, const void *source,
                                 const double *pre, void *scratch, size_t scratch_bytes, void *stream);
int mma_hankel_planes_tc_run(const mma_hankel_problem *p, const mma_hankel_fast_plan_t *plan, const double *ogrid,
                             const double *rgrid, const double *rho, const int64_t *plane_slot, int n_planes,
                             double *planes, void *scratch, size_t scratch_bytes, void *stream);

#ifdef __cplusplus
}
#endif
#endif
