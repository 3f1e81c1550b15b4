/*
 * fftw3.h -- minimal FFTW3 API shim for building the reference TDSE C sources
 * (1DTDSE/sources/tools_fftw3.c) where FFTW is not installed.  Test
 * infrastructure only: it exists so that oracle/_ref can be compiled from the
 * reference sources unchanged.  Only the calls the reference makes are provided
 * (tools_fftw3.c:37-66,115-140): r2c/c2r 1-D plans, execute, destroy, malloc, free.
 * The transforms themselves are oracle/dft.c.
 */
#ifndef MMA_FFTW3_SHIM_H
#define MMA_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct mma_fftw_plan_s *fftw_plan;

#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
