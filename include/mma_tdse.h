/*
 * mma_tdse.h -- C-ABI of the GB300 TDSE library (libmma_gb300.so).
 *
 * Two surfaces:
 *
 * 1. The legacy surface: exactly the symbols and record layouts that the
 *    reference DLL exports and that its Python host binds
 *    (1DTDSE/PythonTDSE.py:48-220, structures 1DTDSE/sources/structures.h:16-147).
 *    A host that loads this library instead of libsingleTDSE.so runs the CUDA
 *    kernels with no other change.  Arrays are host memory allocated with calloc,
 *    as in the reference, and freed by the destructors below.  Unlike the
 *    reference these calls never exit() or print-and-continue: a failure leaves
 *    outputs untouched (or zeroed) and records a status, read back with
 *    mma_last_error() / mma_last_error_message() (thread-local).
 *
 * 2. The batched device surface (mma_tdse_*): many instances, device pointers
 *    (e.g. torch tensors' data_ptr), caller-allocated buffers, a CUDA stream.
 *    Every call returns an mma_status.
 */
#ifndef MMA_TDSE_H
#define MMA_TDSE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Status codes                                                               */
/* ------------------------------------------------------------------------- */
typedef enum {
    MMA_OK = 0,
    MMA_ERR_ARG = 1,          /* invalid argument (sizes, NaN/inf inputs, null pointers) */
    MMA_ERR_GS_NOCONV = 2,    /* ground state did not reach |dE| <= CV within max_iter (reference: exit) */
    MMA_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    MMA_ERR_DFT = 4,          /* a device DFT could not be planned (tables not allocated, or its first
                                 call for a length came while the stream was being captured) */
    MMA_ERR_TOO_LARGE = 5,    /* grid does not fit the selected kernel's limits */
    MMA_ERR_NO_DEVICE = 6,    /* no CUDA device: there is no CPU fallback */
    MMA_ERR_UNSUPPORTED = 7,  /* option the reference accepts but never implemented (velocity gauge) */
    MMA_ERR_TIMEOUT = 8       /* a bounded wait inside a kernel gave up (the kernel returned early) */
} mma_status;

/* ------------------------------------------------------------------------- */
/* Legacy records (byte-identical to 1DTDSE/sources/structures.h:16-147)      */
/* ------------------------------------------------------------------------- */
typedef struct Efield_var {
    double *tgrid;
    double *Field;
    double dt;
    double omega;
    double E0;
    double phi;
    double ton;
    double toff;
    int Nt;
    int nc;
} Efield_var;

typedef struct trg_def {
    double a;
} trg_def;

typedef struct analy_def {
    double tprint;
    int writewft;
} analy_def;

typedef struct output_print_def {
    int Efield;
    int FEfield;
    int sourceterm;
    int Fsourceterm;
    int FEfieldM2;
    int FsourceTermM2;
    int PopTot;
    int tgrid;
    int omegagrid;
    int PopInt;
    int expval_x;
} output_print_def;

typedef struct inputs_def {
    struct trg_def trg;
    struct Efield_var Efield;
    double Eguess;
    double Einit;
    double tmin;
    int Nt;
    int num_t;
    double dt;
    int num_r;
    double dx;
    double *psi0;
    double *x;
    int gauge;
    double x_int;
    struct analy_def analy;
    int InterpByDTorNT;
    int Ntinterp;
    struct output_print_def Print;
    double CV;
    char precision[2];
} inputs_def;

typedef struct outputs_def {
    double *tgrid;
    double *Efield;
    double *sourceterm;
    double *omegagrid;
    double *FEfield;
    double *Fsourceterm;
    double *FEfieldM2;
    double *FsourcetermM2;
    double *PopTot;
    double *PopInt;
    double *expval;
    int Nt;
    int Nomega;
    double **psi;
} outputs_def;

/* ------------------------------------------------------------------------- */
/* Legacy entry points                                                         */
/* ------------------------------------------------------------------------- */

/* Replaces Initialise_grid_and_ground_state (1DTDSE/sources/tools.c:31; bound at
 * PythonTDSE.py:58-61).  Allocates in->x (num_r+1) and in->psi0 (2(num_r+1)),
 * fills the grid and the ground state by inverse iteration on the GPU, sets
 * in->Einit.  Non-convergence within 1000 iterations sets MMA_ERR_GS_NOCONV. */
void Initialise_grid_and_ground_state(inputs_def *in);

/* Replaces call1DTDSE (1DTDSE/sources/singleTDSE.c:28; bound at PythonTDSE.py:75-78).
 * Reads in->Efield (set_time_and_field), in->psi0, in->x; allocates and fills every
 * output array of *out like the reference (lengths Nt+2, Nomega, 2 Nomega), and
 * out->psi when in->analy.writewft is set.  Updates in->Efield.dt, in->num_t and
 * in->Ntinterp as the reference does. */
void call1DTDSE(inputs_def *in, outputs_def *out);

/* Replaces set_time_and_field (1DTDSE/sources/tools.c:423; PythonTDSE.py:216-220):
 * copies N samples of time and field into calloc'ed in->Efield.tgrid / .Field. */
void set_time_and_field(inputs_def *in, double *time, double *field, int N);

/* Replace Set_all_prints / Initialise_Printing_struct (structures.c:92,116). */
output_print_def Set_all_prints(void);
output_print_def Initialise_Printing_struct(void);

/* Replace outputs_destructor / inputs_destructor (structures.c:15,55), free_arr
 * (tools.c:408) and free_mtrx (structures.c:76).  Same ownership rules. */
void outputs_destructor(outputs_def *out);
void inputs_destructor(inputs_def *in);
void free_arr(double *buf);
void free_mtrx(double **buf, int n_rows);

/* Replace window_analysis (tools.c:206-316; PythonTDSE.py:80-109): photoelectron spectrum of
 * psi (2(num_r+1) doubles, interleaved) by the resolvent window method on num_E energies
 * E_start + i Estep with window dE; returns a malloc'ed [num_E] array (free_arr).  The inputs
 * record is passed by value as in the reference; uses num_r, dx and trg.a.  Computed on the GPU
 * (mma_tdse_pes); NULL with the status set on failure. */
double *window_analysis(inputs_def inputs, double *psi, int num_E, double dE, double Estep, double E_start);

/* Replace GaborTransform (tools_fftw3.c:158-213; PythonTDSE.py:111-150): |Gabor transform| of
 * N samples at dt for N_G window centres t_min + i (t_max - t_min)/N_G with width a, the first
 * N_freq DFT bins; returns malloc'ed rows [N_G][N_freq] (free_mtrx).  Computed on the GPU
 * (mma_gabor). */
double **GaborTransform(double *signal, double dt, int N, int N_freq, int N_G, double t_min, double t_max, double a);

/* Status of the last legacy call on this thread (no reference counterpart). */
int mma_last_error(void);
const char *mma_last_error_message(void);

/* ------------------------------------------------------------------------- */
/* Batched device surface                                                      */
/* ------------------------------------------------------------------------- */

/* Threads per CTA of the TDSE kernels; the per-grid tables are laid out for it. */
#define MMA_TDSE_THREADS 256

/* One spatial grid (soft-Coulomb target, spacing, time step).  All pointers are
 * device pointers to caller-allocated memory; sizes follow from n and m:
 *   n   = num_r + 1 sites,  m = ceil(n / MMA_TDSE_THREADS) sites per thread,
 *   L   = m * MMA_TDSE_THREADS (padded length)
 *   x        [n]           grid x_k = k dx - num_r dx / 2        (written by build)
 *   gv       [n]           -dV/dx = x (a^2+x^2)^-3/2              (written by build)
 *   psi0     [2n]          ground state, interleaved re/im       (written by build)
 *   cn_tab   [14 L]        Crank-Nicolson solve tables (complex)  (written by build)
 *   gs_tab   [5 L]         ground-state solve tables (real)       (written by build)
 *   result   [4]           {Einit, iterations, status, |dE| at stop}
 *   c64_tab  [4 * 256 * m32] floats, tables of the complex64 form (precision 1), laid
 *            out for m32 = ceil(m/8)*8 <= 48 sites per thread; NULL when unused
 *            (written by mma_tdse_build_c64_tables)
 *   adj_tab  [10 L] doubles, solve tables of A^H for the adjoint (NULL when unused;
 *            written by mma_tdse_build_grids when not NULL)
 *   c64_threads  CTA size the c64 tables are laid out for: 0 or 256 (m32 <= 48),
 *            512 (m32 8 or 16) or 1024 (m32 8); c64_tab then holds 4 * c64_threads * m32 floats
 *   df_tab   [28 L] floats, the cn_tab entries split into (hi, lo) float pairs for the
 *            float-float form (precision 2); NULL when unused (written by mma_tdse_build_df_tables)
 * The record has 8-byte fields only, so its layout is the same in every ABI. */
typedef struct mma_tdse_grid {
    int64_t n, m;
    double dx, trg_a, dt, x_int, Eguess, CV;
    int64_t max_iter;
    double *x, *gv, *psi0, *cn_tab, *gs_tab, *result;
    int64_t m32;
    float *c64_tab;
    double *adj_tab;
    int64_t c64_threads;
    float *df_tab;
} mma_tdse_grid;

/* One TDSE instance of a batch (offsets are in doubles). */
typedef struct mma_tdse_instance {
    int64_t grid;        /* index into the grid array */
    int64_t n_steps;     /* propagation steps S = k1 * n_field_raw + 2 (the reference's outputs.Nt) */
    int64_t field_off;   /* this instance's refined field samples in buffers.fields */
    int64_t n_field;     /* refined field samples (k1 * n_field_raw); later samples read as 0 */
    int64_t out_off;     /* six series of S+1 doubles: tgrid|Efield|sourceterm|PopTot|PopInt|expval */
    int64_t psi_off;     /* final wavefunction (2n doubles) in buffers.psi_final, or -1 */
    int64_t snap_off;    /* wavefunction snapshots (n_snap x 2n) in buffers.snapshots, or -1 */
    int64_t snap_every;  /* snapshot after step k when k % snap_every == 0 (prop.c:248-263) */
    int64_t n_snap;      /* snapshots kept; the last slot always holds the final state */
    double tmin;         /* start time (the reference's inputs.tmin) */
    double gate_floor;   /* |f| <= gate_floor counts as 0 in the zero-gate test (0 = exact) */
    int64_t ckpt_off;    /* adjoint checkpoints: state psi_{cK} for c = 0, 1, ... (2n doubles each)
                            in buffers.snapshots from this offset, or -1 */
    int64_t ckpt_every;  /* K: steps between checkpoints (0 = none) */
} mma_tdse_instance;

typedef struct mma_tdse_buffers {
    const double *fields;  /* device */
    double *outputs;       /* device */
    double *psi_final;     /* device or NULL */
    double *snapshots;     /* device or NULL */
    int *counter;          /* device int: work-queue head, zeroed by the call on its stream */
    void *scratch;         /* device, mma_tdse_scratch_bytes() bytes */
    size_t scratch_bytes;
} mma_tdse_buffers;

/* Build x, -V', ground state and the solve tables of n_grids grids (device array
 * `grids_dev`, host copy `grids_host` for validation).  One CTA per grid.
 * mode 0: everything; mode 1: CN tables only, from the x and psi0 already in the
 * grid's buffers (a caller-supplied ground state). */
int mma_tdse_build_grids(const mma_tdse_grid *grids_dev, const mma_tdse_grid *grids_host, int n_grids, int mode,
                         void *stream);

/* Build the complex64-form tables of n_grids grids from their FP64 data (after
 * mma_tdse_build_grids): 1/(2 beta) of the FP64 factorisation (half of 1/beta, an exact
 * scaling), V_j and the (real) ground state, rounded once to FP32 and laid out for
 * c64_threads threads x m32 sites per thread (m32 <= 48). */
int mma_tdse_build_c64_tables(const mma_tdse_grid *grids_dev, const mma_tdse_grid *grids_host, int n_grids,
                              void *stream);

/* Propagate n_inst instances in one persistent launch (one CTA per instance at a
 * time, instances pulled from a device work queue).
 *   max_m      largest grid m in the batch (sizes shared memory and scratch)
 *   grid_ctas  persistent CTAs to launch (0 = as many as are resident at once)
 *   precision  0 = FP64, the reference's arithmetic;
 *              1 = complex64 propagation (FP32 wavefunction and sweeps) with the
 *                  factorisation computed in FP64 and the observables summed with
 *                  compensation and finished in FP64; needs c64 tables (n <= 8192);
 *              2 = float-float propagation: the FP64 step and tables carried in double-word
 *                  FP32 arithmetic (about 48 significant bits); needs df tables; psi lives in
 *                  the scratch next to the sweep buffer (mma_tdse_scratch_bytes accounts for it) */
int mma_tdse_propagate(const mma_tdse_instance *insts, int n_inst, const mma_tdse_grid *grids,
                       const mma_tdse_buffers *bufs, int max_m, int grid_ctas, int precision, void *stream);

/* mma_tdse_propagate with the CTA size of the complex64 form chosen by the caller (0 = 256):
 * every instance's grid must carry c64 tables of shape (cta_threads, max_m), see
 * mma_tdse_grid.c64_threads; instances whose grid has another shape get NaN outputs.
 * max_m = 0 (complex64, cta_threads 0 or 256) launches the width-dispatching kernel: the
 * instances' grids may have tables of any 256-thread width (8 to 48 sites per thread), all in
 * one launch from one work queue (one CTA per SM); grids laid out for other CTA sizes get NaN.
 * For precisions 0 and 2 cta_threads must be 0 or 256. */
int mma_tdse_propagate_ex(const mma_tdse_instance *insts, int n_inst, const mma_tdse_grid *grids,
                          const mma_tdse_buffers *bufs, int max_m, int cta_threads, int grid_ctas, int precision,
                          void *stream);

/* Split the FP64 solve tables of n_grids grids (after mma_tdse_build_grids) into the (hi, lo)
 * float pairs of the float-float form: every grid needs df_tab (28 L floats). */
int mma_tdse_build_df_tables(const mma_tdse_grid *grids_dev, const mma_tdse_grid *grids_host, int n_grids,
                             void *stream);

/* 1 if the complex64 form has a kernel for CTA size cta_threads (0 = 256) and m32 sites per thread. */
int mma_tdse_c64_shape_ok(int cta_threads, int m32);

/* No counterpart in the reference.  Persistent CTAs of the complex64 form for tables of that
 * shape: the SMs times the CTAs of that kernel resident per SM (two for 256 threads with
 * m32 <= 16, one otherwise); 0 for a shape without a kernel. */
int mma_tdse_c64_default_ctas(int m32, int cta_threads);

/* Photoelectron spectra on the GPU (window_analysis's algorithm, device pointers): one thread
 * per energy, two FP64 Numerov-tridiagonal solves each.  psi [2(num_r+1)] interleaved, pes
 * [num_E].  Scratch: the energies run in chunks of as many as the scratch holds;
 * mma_tdse_pes_scratch_bytes(num_r, chunk) is the size for `chunk` energies at a time. */
size_t mma_tdse_pes_scratch_bytes(int num_r, int chunk);
int mma_tdse_pes(const double *psi, int num_r, double dx, double trg_a, int num_E, double dE, double Estep,
                 double E_start, double *pes, void *scratch, size_t scratch_bytes, void *stream);

/* Gabor transforms of n_sig signals (GaborTransform's algorithm, device pointers): signal s
 * starts at signals + s * stride (N samples at dt); gabor [n_sig][N_G][N_freq]. */
size_t mma_gabor_scratch_bytes(int n_sig, int N, int N_G);
int mma_gabor(const double *signals, int64_t stride, int n_sig, double dt, int N, int N_freq, int N_G, double t_min,
              double t_max, double a, double *gabor, void *scratch, size_t scratch_bytes, void *stream);

/* Scratch bytes mma_tdse_propagate needs for these arguments. */
size_t mma_tdse_scratch_bytes(int max_m, int grid_ctas, int precision);

/* Persistent CTAs mma_tdse_propagate launches when grid_ctas is 0. */
int mma_tdse_default_ctas(int max_m, int precision);

/* No counterpart in the reference.  The same FP64 propagation as mma_tdse_propagate
 * for callers that cannot allocate device memory (their process's device memory is
 * owned by another runtime's allocator, or they must not allocate while recording a
 * graph): the work space comes from a fixed 8 MiB array compiled into this library
 * (mma_tdse_noalloc_capacity_bytes()), which every GPU that loads the library holds
 * until the process exits.  The caller still passes inputs and outputs.
 *   - The first call on each device looks up that device's address of the array;
 *     make it before any stream capture on that device.  The address is kept for the
 *     life of the process: after cudaDeviceReset (or any teardown of the device's
 *     primary context) it is stale, and this entry point must not be called again in
 *     that process.
 *   - An instance whose grid has more than max_m sites per thread (grid.m > max_m) is
 *     skipped by the kernel and its outputs are NaN; the others run normally.
 *   - Limits: the wavefunction must fit in shared memory and one CTA's sweep buffer
 *     (max_m * 4096 bytes) must fit in the array; larger grids return
 *     MMA_ERR_TOO_LARGE without launching.  Fewer CTAs run when the array is the limit.
 *   - Every call shares the array: calls whose kernels overlap on the GPU (different
 *     streams without ordering) race on it and give wrong results.  Issue them in order.
 *   - Allocates nothing: no cudaMalloc/cudaFree and no allocating library call. */
int mma_tdse_propagate_noalloc(const mma_tdse_instance *insts, int n_inst, const mma_tdse_grid *grids,
                               const double *fields, double *outputs, double *psi_final, double *snapshots,
                               int max_m, void *stream);

/* Size in bytes of the fixed work-space array behind mma_tdse_propagate_noalloc. */
size_t mma_tdse_noalloc_capacity_bytes(void);

/* ------------------------------------------------------------------------- */
/* Adjoint (gradient of a spectral yield with respect to the field)            */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference (the differentiable form).  For each instance the loss
 *   L = dt^2/(2 pi) sum_{q in Q} |DFT_q(s)|^2,  s = sourceterm samples 0..S-1,
 *   Q = {q : w_lo <= 2 pi q / tmax <= w_hi}
 * (the FsourcetermM2 values of the reference's spectrum summed over a band).
 * mma_tdse_loss_grad: L and a_n = dL/ds_n for each instance, from the sourceterm series
 *   in `outputs` (layout of mma_tdse_propagate); loss [n_inst], a [sum(S+1)] at the
 *   instances' out_off/6 ... see a_off; tmax per instance.
 * mma_tdse_adjoint: dL/dF_k for k = 0..S-1 (F_k = the gated field of step k) by the
 *   adjoint Crank-Nicolson recursion, backwards from the last step, recomputing the
 *   forward states between the checkpoints the forward pass stored (instance.ckpt_*).
 *   Grids need adj_tab.  FP64.  grad [sum S] at grad_off[i]; scratch from
 *   mma_tdse_adjoint_scratch_bytes. */
int mma_tdse_loss_grad(const mma_tdse_instance *insts, int n_inst, const double *outputs, const double *tmax,
                       double dt, double w_lo, double w_hi, double *loss, double *a, const int64_t *a_off,
                       void *stream);
size_t mma_tdse_adjoint_scratch_bytes(int max_m, int max_ckpt_every, int grid_ctas);
int mma_tdse_adjoint(const mma_tdse_instance *insts, int n_inst, const mma_tdse_grid *grids,
                     const mma_tdse_buffers *bufs, const double *a, const int64_t *a_off, double *grad,
                     const int64_t *grad_off, int max_m, int max_ckpt_every, int grid_ctas, void *stream);

/* Fourier interpolation (1DTDSE/sources/tools_fftw3.c:24-68) of n_batch fields of
 * equal length n_raw (rows of `raw`, contiguous) by factor k1 into `interp`
 * (k1*n_raw per row): real DFT, zero padding, inverse DFT, 1/n_raw (this library's own DFTs:
 * Stockham mixed radix, Bluestein's convolution for lengths that are not 7-smooth).  The first
 * call for each field length plans its DFTs (device tables, a timed choice of CTA size) and must
 * come before any stream capture; later calls, and mma_tdse_spectra's, are capturable.
 * For k1 = 1 the interpolation is the identity and the samples are copied
 * exactly (the reference's round trip only adds round-off). */
int mma_tdse_prepare_fields(const double *raw, int n_batch, int n_raw, int k1, double *interp, void *stream);

/* Spectra of the sourceterm and Efield series (tools_fftw3.c:84-143) for n_batch
 * instances with equal n_out (= n_steps): omega [n_omega], F [2 n_omega] and
 * M2 [n_omega] for each row; series are read at stride `series_stride`. */
int mma_tdse_spectra(const double *series, int64_t series_stride, int n_batch, int n_out, double dt, double tmax,
                     double *fsig, int64_t fsig_stride, double *fm2, int64_t fm2_stride, double *omega, void *stream);

/* Batched real DFTs in FP64 with FFTW's conventions, the transforms FFTW performs inside the
 * reference's tools_fftw3.c (FourInterp :24-68, calcFFTW3 :84-143, GaborTransform :158-213); this
 * library uses them for all three.  Device pointers; rows at the given strides (in elements).
 *   mma_dft_r2c: X_k = sum_j x_j e^{-2 pi i j k/n}, k = 0 .. n/2 (X interleaved re, im).
 *   mma_dft_c2r: x_j = scale sum_{k<n} X_k e^{+2 pi i j k/n} with X_{n-k} = conj(X_k), from the
 *     first n_bins bins of each row (the rest are zero).
 * The first call for a length n plans it on the current device (tables, and the CTA size picked
 * by timing the candidates on a probe batch) and must come before any stream capture.
 * mma_dft_plan_info reports a length's plan: FFT length (n/2 for even n, n for odd n, or the
 * Bluestein convolution length), whether Bluestein is used, the CTA size (0: the global-memory
 * path for FFT lengths above 7168) and the probe times of the 256- and 512-thread kernels. */
int mma_dft_r2c(int n, const double *x, int64_t x_stride, double *X, int64_t X_stride, int n_batch, void *stream);
int mma_dft_c2r(int n, const double *X, int64_t X_stride, int n_bins, double *x, int64_t x_stride, int n_batch,
                double scale, void *stream);
int mma_dft_plan_info(int n, int *fft_len, int *bluestein, int *cta_threads, float *probe_ms);

#ifdef __cplusplus
}
#endif
#endif
