/* tdse_oracle.h -- CPU restatement of the reference 1D-TDSE (test infrastructure; see tdse_oracle.c). */
#ifndef MMA_TDSE_ORACLE_H
#define MMA_TDSE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_OK = 0, ORACLE_ERR_ARG = 1, ORACLE_ERR_GS_NOCONV = 2 };

typedef struct {
    int num_r;           /* grid has num_r + 1 points */
    double dx, trg_a, x_int;
    const double *x;     /* num_r + 1 */
    const double *psi0;  /* 2 (num_r + 1), interleaved re/im */
    int n_field;
    const double *tgrid_f, *field_f; /* n_field samples */
    double dt_req;
    int interp_by_dt_or_nt, ntinterp;
    double tmin;
    int writewft;
    double tprint;
} oracle_tdse_args;

typedef struct {
    /* time series: n_out + 1 entries written (index 0 .. n_out) */
    double *tgrid, *efield, *sourceterm, *poptot, *popint, *expval;
    /* spectra: n_omega entries (complex ones interleaved, 2 n_omega doubles) */
    double *omegagrid, *fsource, *fsource_m2, *fefield, *fefield_m2;
    double *psi_final; /* optional, 2 (num_r + 1) */
    double *psi_snap;  /* optional, n_snap x 2 (num_r + 1) */
    int n_out, n_omega, k1, n_snap;
    double dt;
} oracle_tdse_result;

int oracle_ground_state(int num_r, double dx, double trg_a, double Eguess, double CV, int max_iter,
                        double *x, double *psi0, double *Einit, int *iters);
int oracle_tdse_sizes(int n_field, const double *tgrid_f, double dt_req, int interp_by_dt_or_nt, int ntinterp,
                      int *k1, double *dt, int *n_out, int *n_omega);
int oracle_propagate(const oracle_tdse_args *in, oracle_tdse_result *out);

#ifdef __cplusplus
}
#endif
#endif
