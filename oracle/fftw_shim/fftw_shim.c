/* fftw_shim.c -- FFTW3 plan/execute calls mapped onto oracle/dft.c (test infrastructure). */
#include <stdlib.h>

#include "fftw3.h"
#include "../dft.h"

struct mma_fftw_plan_s {
    int n;
    int kind; /* 0 = r2c, 1 = c2r */
    double *real;
    double *cplx;
};

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags)
{
    (void)flags;
    fftw_plan p = malloc(sizeof(*p));
    p->n = n;
    p->kind = 0;
    p->real = in;
    p->cplx = (double *)out;
    return p;
}

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags)
{
    (void)flags;
    fftw_plan p = malloc(sizeof(*p));
    p->n = n;
    p->kind = 1;
    p->real = out;
    p->cplx = (double *)in;
    return p;
}

void fftw_execute(const fftw_plan p)
{
    if (p->kind == 0)
        odft_r2c(p->n, p->real, p->cplx);
    else
        odft_c2r(p->n, p->cplx, p->real);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

void *fftw_malloc(size_t n) { return malloc(n); }

void fftw_free(void *p) { free(p); }
