/* dft.h -- oracle-side DFTs (test infrastructure; see dft.c). */
#ifndef MMA_ORACLE_DFT_H
#define MMA_ORACLE_DFT_H

#ifdef __cplusplus
extern "C" {
#endif

/* Complex DFT of length n on interleaved (re,im) data; sign -1 forward, +1 backward; unnormalised. */
void odft_complex(int n, const double *in, double *out, int sign);
/* Real-to-complex forward DFT: n reals in, n/2+1 interleaved complex out. */
void odft_r2c(int n, const double *in, double *out);
/* Complex-to-real backward DFT: n/2+1 interleaved complex in, n reals out; unnormalised. */
void odft_c2r(int n, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
