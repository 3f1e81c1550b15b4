/*
 * dft.c -- CPU discrete Fourier transforms for the oracle (test infrastructure only).
 *
 * This file is part of the oracle: it is linked into the CPU restatement of the
 * TDSE (oracle/tdse_oracle.c) and into the FFTW-API shim that lets the reference
 * C sources compile without FFTW (oracle/fftw_shim).  Nothing in the product
 * path (mma_gb300/) links or calls it.
 *
 * Conventions follow FFTW3's unnormalised transforms, which is what the reference
 * calls (1DTDSE/sources/tools_fftw3.c:41,60,123):
 *   forward   X[k] = sum_n x[n] exp(-2 pi i k n / N)
 *   backward  x[n] = sum_k X[k] exp(+2 pi i k n / N)
 * Arbitrary N is handled by Bluestein's chirp-z algorithm (L. Bluestein, 1970)
 * on top of an iterative radix-2 Cooley-Tukey FFT; power-of-two N goes straight
 * to radix-2.  Chirp phases use the exact integer residue n^2 mod 2N so that the
 * argument of every exp() stays in [0, 2 pi).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "dft.h"

static const double kTwoPi = 6.283185307179586476925286766559;
static const double kPi = 3.141592653589793238462643383279;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* In-place radix-2 FFT on interleaved complex data of length m (power of two). */
static void fft_pow2(double *z, int m, int sign)
{
    /* bit reversal */
    for (int i = 1, j = 0; i < m; i++) {
        int bit = m >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = z[2 * i], ti = z[2 * i + 1];
            z[2 * i] = z[2 * j];
            z[2 * i + 1] = z[2 * j + 1];
            z[2 * j] = tr;
            z[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= m; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; k++) {
            double ang = sign * kTwoPi * (double)k / (double)len;
            double wr = cos(ang), wi = sin(ang);
            for (int s = 0; s < m; s += len) {
                double *a = z + 2 * (s + k), *b = z + 2 * (s + k + half);
                double br = b[0] * wr - b[1] * wi;
                double bi = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br;
                b[1] = a[1] - bi;
                a[0] += br;
                a[1] += bi;
            }
        }
    }
}

void odft_complex(int n, const double *in, double *out, int sign)
{
    if (n <= 0) return;
    if (is_pow2(n)) {
        memmove(out, in, sizeof(double) * 2 * (size_t)n);
        fft_pow2(out, n, sign);
        return;
    }
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    double *chirp = malloc(sizeof(double) * 2 * (size_t)n);
    double *a = calloc(2 * (size_t)m, sizeof(double));
    double *g = calloc(2 * (size_t)m, sizeof(double));
    const int64_t two_n = 2 * (int64_t)n;
    for (int k = 0; k < n; k++) {
        /* chirp_k = exp(sign * i pi k^2 / n), phase reduced exactly mod 2n */
        int64_t r = ((int64_t)k * (int64_t)k) % two_n;
        double ang = sign * kPi * (double)r / (double)n;
        chirp[2 * k] = cos(ang);
        chirp[2 * k + 1] = sin(ang);
    }
    for (int k = 0; k < n; k++) {
        /* a_k = x_k * chirp_k ; g_k = conj(chirp_k) (symmetric in k) */
        double xr = in[2 * k], xi = in[2 * k + 1];
        double cr = chirp[2 * k], ci = chirp[2 * k + 1];
        a[2 * k] = xr * cr - xi * ci;
        a[2 * k + 1] = xr * ci + xi * cr;
        g[2 * k] = cr;
        g[2 * k + 1] = -ci;
        if (k > 0) {
            g[2 * (m - k)] = cr;
            g[2 * (m - k) + 1] = -ci;
        }
    }
    fft_pow2(a, m, -1);
    fft_pow2(g, m, -1);
    for (int k = 0; k < m; k++) {
        double ar = a[2 * k], ai = a[2 * k + 1];
        double gr = g[2 * k], gi = g[2 * k + 1];
        a[2 * k] = ar * gr - ai * gi;
        a[2 * k + 1] = ar * gi + ai * gr;
    }
    fft_pow2(a, m, +1);
    const double inv_m = 1.0 / (double)m;
    for (int k = 0; k < n; k++) {
        double yr = a[2 * k] * inv_m, yi = a[2 * k + 1] * inv_m;
        double cr = chirp[2 * k], ci = chirp[2 * k + 1];
        out[2 * k] = yr * cr - yi * ci;
        out[2 * k + 1] = yr * ci + yi * cr;
    }
    free(chirp);
    free(a);
    free(g);
}

void odft_r2c(int n, const double *in, double *out)
{
    double *z = malloc(sizeof(double) * 2 * (size_t)n);
    double *y = malloc(sizeof(double) * 2 * (size_t)n);
    for (int k = 0; k < n; k++) {
        z[2 * k] = in[k];
        z[2 * k + 1] = 0.0;
    }
    odft_complex(n, z, y, -1);
    memcpy(out, y, sizeof(double) * 2 * (size_t)(n / 2 + 1));
    free(z);
    free(y);
}

void odft_c2r(int n, const double *in, double *out)
{
    /* Hermitian extension; like FFTW, the imaginary parts of the DC term and
     * (for even n) of the Nyquist term are ignored. */
    double *z = calloc(2 * (size_t)n, sizeof(double));
    double *y = malloc(sizeof(double) * 2 * (size_t)n);
    int nc = n / 2 + 1;
    z[0] = in[0];
    for (int k = 1; k < nc; k++) {
        if (2 * k == n) {
            z[2 * k] = in[2 * k];
            continue;
        }
        z[2 * k] = in[2 * k];
        z[2 * k + 1] = in[2 * k + 1];
        z[2 * (n - k)] = in[2 * k];
        z[2 * (n - k) + 1] = -in[2 * k + 1];
    }
    odft_complex(n, z, y, +1);
    for (int k = 0; k < n; k++) out[k] = y[2 * k];
    free(z);
    free(y);
}
