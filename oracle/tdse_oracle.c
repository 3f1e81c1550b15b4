/*
 * tdse_oracle.c -- CPU restatement of the reference 1D-TDSE (MMA 1DTDSE/sources).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, smoke() and
 * bench.py's CPU-baseline leg call it to check (or time beside) the CUDA path.
 * The product library (mma_gb300/csrc) never links or calls it.
 *
 * Pinned against the reference itself: tests build the reference DLL sources
 * unchanged (oracle/Makefile -> oracle/_ref/libsingleTDSE.so, with the FFTW
 * shim) and compare this restatement with it; the golden fixtures under tests/golden hold outputs of
 * that build for the GPU machine, where the reference sources are absent.
 *
 * The algorithm, step by step, with the reference lines it follows:
 *   grid             x_k = k dx - num_r dx / 2                    tools.c:62-79
 *   potential        V = -1/sqrt(a^2 + x^2), -V' = x (a^2+x^2)^-3/2  tools.c:91-113
 *   ground state     shifted inverse iteration (H - Eg M2)^-1 M2 psi,
 *                    normalise, Numerov energy quotient, |dE| <= CV   tridiag.c:86-238,251-274
 *   time grid        dt refinement k1, Fourier interpolation       singleTDSE.c:50-75, tools_fftw3.c:24-68
 *   one step         CN-Numerov: (M2 + i dt/2 K) psi' = (M2 - i dt/2 K) psi,
 *                    K = T + M2 V; Thomas solve; phase exp(+i E dt x)  prop.c:115-205, tridiag.c:26-70
 *   observables      |<psi0|psi>|^2, window population, <x>,
 *                    -<V'> + E                                      prop.c:293-347
 *   spectra          dt/sqrt(2 pi) conj(DFT), dt^2/(2 pi)|DFT|^2    tools_fftw3.c:84-143
 * The length gauge is the only reachable gauge (prop.c:197; the velocity branch
 * has A = 0 and is forced off by the reference drivers).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dft.h"
#include "tdse_oracle.h"

static const double kPi = 3.141592653589793238462643383279;

typedef struct {
    double re, im;
} cplx;

static inline double soft_coulomb(double x, double a) { return -1.0 / sqrt(a * a + x * x); }
static inline double minus_grad_v(double x, double a) { return x * pow(a * a + x * x, -1.5); }

/* Thomas elimination without pivoting on a complex tridiagonal system; row j
 * reads sub[j-1], diag[j], sup[j] like tridiag.c:26-70 does. */
static void thomas(int n, const cplx *sub, const cplx *diag, const cplx *sup, const cplx *rhs,
                   cplx *u, cplx *work)
{
    cplx beta = diag[0];
    double bn = beta.re * beta.re + beta.im * beta.im;
    u[0].re = (rhs[0].re * beta.re + rhs[0].im * beta.im) / bn;
    u[0].im = (rhs[0].im * beta.re - rhs[0].re * beta.im) / bn;
    for (int j = 1; j < n; j++) {
        cplx c = sup[j - 1], a = sub[j - 1];
        cplx g = {(c.re * beta.re + c.im * beta.im) / bn, (c.im * beta.re - c.re * beta.im) / bn};
        work[j] = g;
        beta.re = diag[j].re - (a.re * g.re - a.im * g.im);
        beta.im = diag[j].im - (a.im * g.re + a.re * g.im);
        bn = beta.re * beta.re + beta.im * beta.im;
        double tr = rhs[j].re - a.re * u[j - 1].re + a.im * u[j - 1].im;
        double ti = rhs[j].im - a.re * u[j - 1].im - a.im * u[j - 1].re;
        u[j].re = (tr * beta.re + ti * beta.im) / bn;
        u[j].im = (ti * beta.re - tr * beta.im) / bn;
    }
    for (int j = n - 2; j >= 0; j--) {
        cplx g = work[j + 1], v = u[j + 1];
        u[j].re -= g.re * v.re - g.im * v.im;
        u[j].im -= g.re * v.im + g.im * v.re;
    }
}

/* Numerov mass matrix M2 = tridiag(1, 10, 1)/12 applied to psi. */
static void apply_m2(int n, const cplx *p, cplx *out)
{
    for (int j = 0; j < n; j++) {
        double sr = 10.0 * p[j].re / 12.0, si = 10.0 * p[j].im / 12.0;
        double nr = 0.0, ni = 0.0;
        if (j > 0) {
            nr += p[j - 1].re;
            ni += p[j - 1].im;
        }
        if (j + 1 < n) {
            nr += p[j + 1].re;
            ni += p[j + 1].im;
        }
        out[j].re = sr + nr / 12.0;
        out[j].im = si + ni / 12.0;
    }
}

static double sum_abs2(int n, const cplx *p)
{
    double s = 0.0;
    for (int j = 0; j < n; j++) s += p[j].re * p[j].re + p[j].im * p[j].im;
    return s;
}

static void scale_to_unit_norm(int n, cplx *p)
{
    double nrm = sqrt(sum_abs2(n, p));
    for (int j = 0; j < n; j++) {
        p[j].re /= nrm;
        p[j].im /= nrm;
    }
}

/* Numerov energy quotient <M2 psi | K psi> / <M2 psi | M2 psi>, K = T + M2 V
 * (tridiag.c:172-238, including its real+imag accumulation). */
static double numerov_energy(int n, const cplx *p, const double *v, double inv_dx2)
{
    double e = 0.0, nm = 0.0;
    for (int j = 0; j < n; j++) {
        cplx k, m;
        double nbr_re = 0.0, nbr_im = 0.0, vn_re = 0.0, vn_im = 0.0;
        if (j > 0) {
            nbr_re += p[j - 1].re;
            nbr_im += p[j - 1].im;
            vn_re += p[j - 1].re * v[j - 1];
            vn_im += p[j - 1].im * v[j - 1];
        }
        if (j + 1 < n) {
            nbr_re += p[j + 1].re;
            nbr_im += p[j + 1].im;
            vn_re += p[j + 1].re * v[j + 1];
            vn_im += p[j + 1].im * v[j + 1];
        }
        k.re = inv_dx2 * p[j].re - 0.5 * inv_dx2 * nbr_re + (10.0 / 12.0) * p[j].re * v[j] + vn_re / 12.0;
        k.im = inv_dx2 * p[j].im - 0.5 * inv_dx2 * nbr_im + (10.0 / 12.0) * p[j].im * v[j] + vn_im / 12.0;
        m.re = 10.0 * p[j].re / 12.0 + nbr_re / 12.0;
        m.im = 10.0 * p[j].im / 12.0 + nbr_im / 12.0;
        e += (k.re * m.re + k.im * m.im) + (k.im * m.re - k.re * m.im);
        nm += m.re * m.re + m.im * m.im;
    }
    return e / nm;
}

int oracle_ground_state(int num_r, double dx, double trg_a, double Eguess, double CV, int max_iter,
                        double *x, double *psi0, double *Einit, int *iters)
{
    if (num_r < 2 || !(dx > 0.0)) return ORACLE_ERR_ARG;
    const int n = num_r + 1;
    const double xmax = 0.5 * num_r * dx;
    for (int k = 0; k < n; k++) x[k] = (double)k * dx - xmax;
    double *v = malloc(sizeof(double) * (n + 1));
    for (int k = 0; k < n; k++) v[k] = soft_coulomb(x[k], trg_a);
    v[n] = soft_coulomb(x[n - 1] + (x[n - 1] - x[n - 2]), trg_a);
    const double inv_dx2 = 1.0 / (dx * dx);

    cplx *sub = malloc(sizeof(cplx) * n), *dia = malloc(sizeof(cplx) * n), *sup = malloc(sizeof(cplx) * n);
    cplx *psi = (cplx *)psi0, *rhs = malloc(sizeof(cplx) * n), *res = malloc(sizeof(cplx) * n);
    cplx *work = malloc(sizeof(cplx) * n);
    for (int k = 0; k < n; k++) {
        /* (K - Eg M2) with K = T + M2 V, tridiag.c:101-115 */
        sub[k].re = -0.5 * inv_dx2 - Eguess / 12.0 + v[k] / 12.0;
        sub[k].im = 0.0;
        dia[k].re = 10.0 * v[k] / 12.0 + inv_dx2 - 10.0 * Eguess / 12.0;
        dia[k].im = 0.0;
        sup[k].re = -0.5 * inv_dx2 - Eguess / 12.0 + v[k + 1] / 12.0;
        sup[k].im = 0.0;
        psi[k].re = 1.0; /* tools.c:39-42 */
        psi[k].im = 0.0;
    }
    double e_old = Eguess, energy = Eguess;
    int it = 0, status = ORACLE_OK;
    for (;;) {
        apply_m2(n, psi, rhs);
        thomas(n, sub, dia, sup, rhs, res, work);
        scale_to_unit_norm(n, res);
        memcpy(psi, res, sizeof(cplx) * n);
        energy = numerov_energy(n, res, v, inv_dx2);
        double test = fabs(energy - e_old);
        e_old = energy;
        ++it;
        if (it >= max_iter) {
            status = ORACLE_ERR_GS_NOCONV;
            break;
        }
        if (!(test > CV)) break;
    }
    scale_to_unit_norm(n, psi); /* tridiag.c:150 */
    *Einit = energy;
    if (iters) *iters = it;
    free(v);
    free(sub);
    free(dia);
    free(sup);
    free(rhs);
    free(res);
    free(work);
    return status;
}

int oracle_tdse_sizes(int n_field, const double *tgrid_f, double dt_req, int interp_by_dt_or_nt, int ntinterp,
                      int *k1_out, double *dt_out, int *n_out, int *n_omega)
{
    if (n_field < 2) return ORACLE_ERR_ARG;
    double dt_f = tgrid_f[1] - tgrid_f[0];
    int k1;
    if (interp_by_dt_or_nt == 1) {
        k1 = ntinterp + 1;
    } else {
        k1 = (int)floor(dt_f / dt_req); /* singleTDSE.c:59-62 */
        if (k1 != 1) k1++;
    }
    if (k1 < 1) return ORACLE_ERR_ARG;
    *k1_out = k1;
    *dt_out = dt_f / (double)k1;
    *n_out = k1 * n_field + 2; /* singleTDSE.c:72,94 */
    *n_omega = *n_out / 2 + 1;
    return ORACLE_OK;
}

/* Fourier interpolation by zero padding (tools_fftw3.c:24-68): returns k1*n samples.
 * For k1 = 1 it is the identity in exact arithmetic and the samples are copied: the
 * reference's round trip only adds round-off, whose sign can flip its zero gate on a
 * field that starts at exactly 0. */
static double *fourier_interp(int k1, const double *sig, int n)
{
    if (k1 == 1) {
        double *cp = calloc((size_t)n + 2, sizeof(double));
        memcpy(cp, sig, sizeof(double) * (size_t)n);
        return cp;
    }
    int nc = n / 2 + 1, n2 = k1 * n, nc2 = n2 / 2 + 1;
    double *spec = malloc(sizeof(double) * 2 * nc);
    double *pad = calloc(2 * (size_t)nc2, sizeof(double));
    double *out = calloc((size_t)n2 + 2, sizeof(double));
    odft_r2c(n, sig, spec);
    for (int k = 0; k < nc; k++) {
        pad[2 * k] = spec[2 * k] / n;
        pad[2 * k + 1] = spec[2 * k + 1] / n;
    }
    odft_c2r(n2, pad, out);
    free(spec);
    free(pad);
    return out;
}

static void spectrum(int n, double dt, double tmax, const double *sig, double *omega, double *fsig, double *fm2)
{
    int nc = n / 2 + 1;
    double *spec = malloc(sizeof(double) * 2 * nc);
    odft_r2c(n, sig, spec);
    const double dxi = 2.0 * kPi / tmax, c1 = dt / sqrt(2.0 * kPi), c2 = dt * dt / (2.0 * kPi);
    for (int k = 0; k < nc; k++) {
        if (omega) omega[k] = (double)k * dxi;
        if (fsig) {
            fsig[2 * k] = c1 * spec[2 * k];
            fsig[2 * k + 1] = -c1 * spec[2 * k + 1];
        }
        if (fm2) fm2[k] = c2 * (spec[2 * k] * spec[2 * k] + spec[2 * k + 1] * spec[2 * k + 1]);
    }
    free(spec);
}

/* Index window of findinterval() (tools_algorithmic.c:19-43) for +-x_int. */
static void population_window(int num_r, const double *x, double x_int, int *lo, int *hi)
{
    int i;
    *lo = -1;
    if (!(-x_int < x[0])) {
        for (i = 0; i < num_r; i++)
            if (-x_int <= x[i + 1]) break;
        *lo = (i < num_r) ? i : num_r;
    }
    if (x_int < x[0]) {
        *hi = 0;
    } else {
        for (i = 0; i < num_r; i++)
            if (x_int <= x[i + 1]) break;
        *hi = (i < num_r) ? i + 1 : num_r + 1;
    }
}

int oracle_propagate(const oracle_tdse_args *in, oracle_tdse_result *out)
{
    int k1, n_out, n_omega;
    double dt;
    int st = oracle_tdse_sizes(in->n_field, in->tgrid_f, in->dt_req, in->interp_by_dt_or_nt, in->ntinterp, &k1,
                               &dt, &n_out, &n_omega);
    if (st != ORACLE_OK) return st;
    const int num_r = in->num_r, n = num_r + 1;
    const double dx = in->dx, a = in->trg_a;
    const double tmax = in->tgrid_f[in->n_field - 1] - in->tgrid_f[0];
    const int n_interp = k1 * in->n_field;
    double *f = fourier_interp(k1, in->field_f, in->n_field);
    /* after a genuine interpolation (k1 > 1), samples within round-off of zero count
     * as zero in the gate test */
    double gate_floor = 0.0;
    if (k1 > 1) {
        for (int i = 0; i < in->n_field; i++)
            if (fabs(in->field_f[i]) > gate_floor) gate_floor = fabs(in->field_f[i]);
        gate_floor *= 1e-13;
    }
    /* Samples at and beyond k1*n_field are zero (the reference reads the zero
     * padding of its interpolation buffer there, singleTDSE.c:66 / prop.c:127). */
    const double *x = in->x;
    const cplx *psi0 = (const cplx *)in->psi0;

    double *v = malloc(sizeof(double) * (n + 1));
    double *gv = malloc(sizeof(double) * n);
    for (int j = 0; j < n; j++) {
        v[j] = soft_coulomb(x[j], a);
        gv[j] = minus_grad_v(x[j], a);
    }
    v[n] = soft_coulomb(x[num_r] + dx, a);

    cplx *sub = malloc(sizeof(cplx) * n), *dia = malloc(sizeof(cplx) * n), *sup = malloc(sizeof(cplx) * n);
    cplx *psi = malloc(sizeof(cplx) * n), *rhs = malloc(sizeof(cplx) * n), *sol = malloc(sizeof(cplx) * n);
    cplx *work = malloc(sizeof(cplx) * n);
    memcpy(psi, psi0, sizeof(cplx) * n);

    int lo, hi;
    population_window(num_r, x, in->x_int, &lo, &hi);
    if (lo < 0) lo = 0;
    if (hi > num_r) hi = num_r;
    double pop0 = 0.0;
    for (int j = lo; j <= hi; j++) pop0 += psi0[j].re * psi0[j].re + psi0[j].im * psi0[j].im;

    double tt = in->tmin, field = 0.0;
    out->tgrid[0] = tt;
    out->sourceterm[0] = 0.0;
    out->efield[0] = 0.0;
    out->popint[0] = pop0;
    out->poptot[0] = 1.0;
    out->expval[0] = 0.0;

    const int steps_per_print = in->writewft ? (int)floor(in->tprint / dt) : 1;
    const int n_snap = in->writewft ? n_out / steps_per_print : 0;
    int i_wf = 0;

    const double h = 0.5 * dt, coef = 0.5 * dt / (dx * dx);
    int gate_closed = 1;
    for (int k = 0; k < n_out; k++) {
        tt += dt;
        double fk = (k < n_interp) ? f[k] : 0.0, fk1 = (k + 1 < n_interp) ? f[k + 1] : 0.0;
        if (gate_closed) { /* prop.c:125-134 */
            double ga = fabs(fk) <= gate_floor ? 0.0 : fk, gb = fabs(fk1) <= gate_floor ? 0.0 : fk1;
            if (ga * gb <= 0.0) gate_closed = 0;
            field = 0.0;
        } else {
            field = fk;
        }
        /* LHS M2 + i dt/2 K  (prop.c:138-159) */
        for (int j = 0; j < n; j++) {
            sub[j].re = 1.0 / 12.0;
            sub[j].im = h * (-0.5 / (dx * dx)) + h / 12.0 * v[j];
            dia[j].re = 10.0 / 12.0;
            dia[j].im = h / (dx * dx) + h * 10.0 / 12.0 * v[j];
            sup[j].re = 1.0 / 12.0;
            sup[j].im = h * (-0.5 / (dx * dx)) + h / 12.0 * v[j + 1];
        }
        /* RHS (M2 - i dt/2 K) psi  (prop.c:162-190) */
        for (int j = 0; j < n; j++) {
            double mr = 10.0 / 12.0 * psi[j].re, mi = 10.0 / 12.0 * psi[j].im;
            double kr = coef * psi[j].re + h * 10.0 / 12.0 * v[j] * psi[j].re;
            double ki = coef * psi[j].im + h * 10.0 / 12.0 * v[j] * psi[j].im;
            for (int s = -1; s <= 1; s += 2) {
                int q = j + s;
                if (q < 0 || q >= n) continue;
                mr += psi[q].re / 12.0;
                mi += psi[q].im / 12.0;
                kr += -0.5 * coef * psi[q].re + h / 12.0 * v[q] * psi[q].re;
                ki += -0.5 * coef * psi[q].im + h / 12.0 * v[q] * psi[q].im;
            }
            rhs[j].re = mr + ki;
            rhs[j].im = mi - kr;
        }
        thomas(n, sub, dia, sup, rhs, sol, work);
        /* length-gauge phase exp(+i E dt x)  (prop.c:200-204) */
        for (int j = 0; j < n; j++) {
            double th = field * dt * x[j], c = cos(th), s = sin(th);
            psi[j].re = c * sol[j].re - s * sol[j].im;
            psi[j].im = c * sol[j].im + s * sol[j].re;
        }
        out->tgrid[k + 1] = tt;
        out->efield[k + 1] = field;
        /* observables (prop.c:293-347) */
        double pr = 0.0, pi = 0.0, xs = 0.0, gs = 0.0, win = 0.0;
        for (int j = 0; j < n; j++) {
            pr += psi[j].re * psi0[j].re + psi[j].im * psi0[j].im;
            pi += psi[j].re * psi0[j].im - psi[j].im * psi0[j].re;
        }
        for (int j = lo; j <= hi; j++) win += psi[j].re * psi[j].re + psi[j].im * psi[j].im;
        for (int j = 0; j < n; j++) {
            double d = psi[j].re * psi[j].re + psi[j].im * psi[j].im;
            xs += d * x[j];
        }
        for (int j = 0; j < n; j++) {
            double d = psi[j].re * psi[j].re + psi[j].im * psi[j].im;
            gs += d * gv[j];
        }
        out->sourceterm[k + 1] = -gs + field;
        out->poptot[k + 1] = pr * pr + pi * pi;
        out->expval[k + 1] = xs;
        out->popint[k + 1] = win;
        if (n_snap > 0 && out->psi_snap) { /* prop.c:248-263 */
            if (k % steps_per_print == 0 && i_wf < n_snap - 1) {
                memcpy(out->psi_snap + (size_t)i_wf * 2 * n, psi, sizeof(cplx) * n);
                i_wf++;
            }
            if (k == n_out - 1 && i_wf == n_snap - 1)
                memcpy(out->psi_snap + (size_t)i_wf * 2 * n, psi, sizeof(cplx) * n);
        }
    }
    if (out->psi_final) memcpy(out->psi_final, psi, sizeof(cplx) * n);

    spectrum(n_out, dt, tmax, out->efield, NULL, out->fefield, out->fefield_m2);
    spectrum(n_out, dt, tmax, out->sourceterm, out->omegagrid, out->fsource, out->fsource_m2);
    out->n_out = n_out;
    out->n_omega = n_omega;
    out->k1 = k1;
    out->dt = dt;
    out->n_snap = n_snap;

    free(f);
    free(v);
    free(gv);
    free(sub);
    free(dia);
    free(sup);
    free(psi);
    free(rhs);
    free(sol);
    free(work);
    return ORACLE_OK;
}
