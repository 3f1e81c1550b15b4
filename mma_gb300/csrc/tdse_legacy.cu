// tdse_legacy.cu -- the reference DLL's symbols, running the GPU kernels.
//
// Each legacy call takes and returns host records laid out like
// 1DTDSE/sources/structures.h; inside, it stages the arrays to the GPU, runs the
// batched device surface for one instance, and copies the results back into
// calloc'ed host arrays with the reference's lengths and ownership rules.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/mma_tdse.h"

namespace {

thread_local int g_status = MMA_OK;
thread_local char g_msg[512] = "";

void set_status(int st, const char* fmt, ...)
{
    g_status = st;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

void clear_status()
{
    g_status = MMA_OK;
    g_msg[0] = 0;
}

const double kPi = 3.14159265358979323846;

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_status(MMA_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));             \
            goto fail;                                                                            \
        }                                                                                         \
    } while (0)

bool have_device()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        set_status(MMA_ERR_NO_DEVICE, "no CUDA device is available; this library has no CPU path");
        return false;
    }
    return true;
}

// Device buffers of one grid, carved from a single allocation.
struct DevGrid {
    mma_tdse_grid h{};
    mma_tdse_grid* d = nullptr;
    double* buf = nullptr;
};

void free_grid(DevGrid& g)
{
    if (g.buf) cudaFree(g.buf);
    if (g.d) cudaFree(g.d);
    g.buf = nullptr;
    g.d = nullptr;
}

int alloc_grid(DevGrid& g, int num_r, double dx, double a, double dt, double x_int, double Eguess, double CV)
{
    const int64_t n = (int64_t)num_r + 1, m = (n + MMA_TDSE_THREADS - 1) / MMA_TDSE_THREADS;
    const int64_t L = m * MMA_TDSE_THREADS;
    const size_t nd = (size_t)(n + n + 2 * n + 14 * L + 5 * L + 4);
    if (cudaMalloc((void**)&g.buf, nd * sizeof(double)) != cudaSuccess) return MMA_ERR_CUDA;
    if (cudaMalloc((void**)&g.d, sizeof(mma_tdse_grid)) != cudaSuccess) return MMA_ERR_CUDA;
    double* p = g.buf;
    g.h.n = n;
    g.h.m = m;
    g.h.dx = dx;
    g.h.trg_a = a;
    g.h.dt = dt;
    g.h.x_int = x_int;
    g.h.Eguess = Eguess;
    g.h.CV = CV;
    g.h.max_iter = 1000;  // tridiag.c:139
    g.h.x = p;
    p += n;
    g.h.gv = p;
    p += n;
    g.h.psi0 = p;
    p += 2 * n;
    g.h.cn_tab = p;
    p += 14 * L;
    g.h.gs_tab = p;
    p += 5 * L;
    g.h.result = p;
    g.h.m32 = 0;
    g.h.c64_tab = nullptr;
    g.h.adj_tab = nullptr;
    g.h.c64_threads = 0;
    g.h.df_tab = nullptr;
    if (cudaMemcpy(g.d, &g.h, sizeof(mma_tdse_grid), cudaMemcpyHostToDevice) != cudaSuccess) return MMA_ERR_CUDA;
    return MMA_OK;
}

}  // namespace

extern "C" int mma_last_error(void) { return g_status; }
extern "C" const char* mma_last_error_message(void) { return g_msg; }

// tools.c:31-51
extern "C" void Initialise_grid_and_ground_state(inputs_def* in)
{
    clear_status();
    if (!in || in->num_r < 2 || !(in->dx > 0.0) || !std::isfinite(in->trg.a) || !std::isfinite(in->Eguess)) {
        set_status(MMA_ERR_ARG, "invalid grid parameters (num_r >= 2, dx > 0, finite a and Eguess required)");
        return;
    }
    if (!have_device()) return;
    DevGrid g;
    double res[4] = {0, 0, 0, 0};
    const int64_t n = (int64_t)in->num_r + 1;
    double* x = nullptr;
    double* psi0 = nullptr;
    int rc = alloc_grid(g, in->num_r, in->dx, in->trg.a, in->dt > 0.0 ? in->dt : 0.25, in->x_int, in->Eguess, in->CV);
    if (rc != MMA_OK) {
        set_status(rc, "device allocation failed");
        free_grid(g);
        return;
    }
    rc = mma_tdse_build_grids(g.d, &g.h, 1, 0, nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "grid build launch failed");
        free_grid(g);
        return;
    }
    x = (double*)calloc((size_t)n, sizeof(double));
    psi0 = (double*)calloc(2 * (size_t)n, sizeof(double));
    CK(cudaMemcpy(x, g.h.x, sizeof(double) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(psi0, g.h.psi0, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(res, g.h.result, sizeof(res), cudaMemcpyDeviceToHost));
    in->x = x;
    in->psi0 = psi0;
    in->Einit = res[0];
    if ((int)res[2] != MMA_OK)
        set_status(MMA_ERR_GS_NOCONV, "ground state not converged after %d iterations (|dE| = %g > CV = %g)",
                   (int)res[1], res[3], in->CV);
    free_grid(g);
    return;
fail:
    free(x);
    free(psi0);
    free_grid(g);
}

// singleTDSE.c:28-117
extern "C" void call1DTDSE(inputs_def* in, outputs_def* out)
{
    clear_status();
    if (!in || !out || !in->Efield.tgrid || !in->Efield.Field || in->Efield.Nt < 2 || !in->psi0 || !in->x ||
        in->num_r < 2 || !(in->dx > 0.0)) {
        set_status(MMA_ERR_ARG, "call1DTDSE needs a field (Nt >= 2), a grid and a ground state");
        return;
    }
    if (in->gauge != 0) {
        set_status(MMA_ERR_UNSUPPORTED, "only the length gauge is implemented (the reference marks the velocity "
                                        "gauge NOT IMPLEMENTED)");
        return;
    }
    const int nf = in->Efield.Nt;
    for (int i = 0; i < nf; i++)
        if (!std::isfinite(in->Efield.Field[i]) || !std::isfinite(in->Efield.tgrid[i])) {
            set_status(MMA_ERR_ARG, "field or time grid has a non-finite sample at index %d", i);
            return;
        }
    if (!have_device()) return;

    const double dt_f = in->Efield.tgrid[1] - in->Efield.tgrid[0];
    const double tmax = in->Efield.tgrid[nf - 1] - in->Efield.tgrid[0];
    int k1;
    if (in->InterpByDTorNT == 1) {
        k1 = in->Ntinterp + 1;
    } else {
        k1 = (int)floor(dt_f / in->dt);
        in->Ntinterp = k1;
        if (k1 != 1) k1++;
    }
    if (k1 < 1 || !(dt_f > 0.0) || !(tmax > 0.0)) {
        set_status(MMA_ERR_ARG, "time grid must be increasing and the refinement factor positive");
        return;
    }
    const double dt = dt_f / (double)k1;
    const int nt = k1 * nf + 1;      // singleTDSE.c:72
    const int n_out = nt + 1;        // outputs.Nt
    const int n_om = n_out / 2 + 1;  // tools_fftw3.c:103-104
    in->Efield.dt = dt;
    in->num_t = (int)floor((2 * kPi) / (0.057 * dt)) + 1;

    const int64_t n = (int64_t)in->num_r + 1;
    int n_snap = 0, snap_every = 1;
    if (in->analy.writewft) {
        snap_every = (int)floor(in->analy.tprint / dt);
        if (snap_every < 1) {
            set_status(MMA_ERR_ARG, "tprint shorter than one time step");
            return;
        }
        n_snap = n_out / snap_every;
    }

    DevGrid g;
    double *d_raw = nullptr, *d_fld = nullptr, *d_out = nullptr, *d_spec = nullptr, *d_snap = nullptr;
    void* d_scratch = nullptr;
    int* d_counter = nullptr;
    mma_tdse_instance* d_inst = nullptr;
    const int64_t S1 = (int64_t)n_out + 1;
    std::vector<double> series;
    mma_tdse_instance I{};
    mma_tdse_buffers B{};
    size_t sbytes = 0;
    int rc = alloc_grid(g, in->num_r, in->dx, in->trg.a, dt, in->x_int, in->Eguess, in->CV);
    if (rc != MMA_OK) {
        set_status(rc, "device allocation failed");
        free_grid(g);
        return;
    }
    CK(cudaMemcpy(g.h.x, in->x, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.h.psi0, in->psi0, sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    rc = mma_tdse_build_grids(g.d, &g.h, 1, 1, nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "table build failed");
        goto fail;
    }
    CK(cudaMalloc((void**)&d_raw, sizeof(double) * nf));
    CK(cudaMalloc((void**)&d_fld, sizeof(double) * (size_t)k1 * nf));
    CK(cudaMemcpy(d_raw, in->Efield.Field, sizeof(double) * nf, cudaMemcpyHostToDevice));
    rc = mma_tdse_prepare_fields(d_raw, 1, nf, k1, d_fld, nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "field interpolation failed");
        goto fail;
    }
    CK(cudaMalloc((void**)&d_out, sizeof(double) * 6 * S1));
    CK(cudaMalloc((void**)&d_spec, sizeof(double) * (2 * 2 * n_om + 2 * n_om + n_om)));
    if (n_snap > 0) CK(cudaMalloc((void**)&d_snap, sizeof(double) * 2 * n * (size_t)n_snap));
    CK(cudaMalloc((void**)&d_counter, sizeof(int)));
    I.grid = 0;
    I.n_steps = n_out;
    I.field_off = 0;
    I.n_field = (int64_t)k1 * nf;
    I.out_off = 0;
    I.psi_off = -1;
    I.snap_off = n_snap > 0 ? 0 : -1;
    I.snap_every = snap_every;
    I.n_snap = n_snap;
    I.tmin = in->tmin;
    I.gate_floor = 0.0;
    I.ckpt_off = -1;
    I.ckpt_every = 0;
    if (k1 > 1) {
        double fmax = 0.0;
        for (int i = 0; i < nf; i++) fmax = fmax > fabs(in->Efield.Field[i]) ? fmax : fabs(in->Efield.Field[i]);
        I.gate_floor = 1e-13 * fmax;
    }
    CK(cudaMalloc((void**)&d_inst, sizeof(I)));
    CK(cudaMemcpy(d_inst, &I, sizeof(I), cudaMemcpyHostToDevice));
    sbytes = mma_tdse_scratch_bytes((int)g.h.m, 1, 0);
    CK(cudaMalloc(&d_scratch, sbytes));
    B.fields = d_fld;
    B.outputs = d_out;
    B.psi_final = nullptr;
    B.snapshots = d_snap;
    B.counter = d_counter;
    B.scratch = d_scratch;
    B.scratch_bytes = sbytes;
    rc = mma_tdse_propagate(d_inst, 1, g.d, &B, (int)g.h.m, 1, 0, nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "propagation launch failed");
        goto fail;
    }
    // spectra of Efield (series 1) and sourceterm (series 2): tools_fftw3.c:84-143
    {
        double* fe = d_spec;             // [FEfield | Fsourceterm], 2 n_om doubles each
        double* m2 = d_spec + 4 * n_om;  // [FEfieldM2 | FsourcetermM2]
        double* om = d_spec + 6 * n_om;
        rc = mma_tdse_spectra(d_out + 1 * S1, S1, 2, n_out, dt, tmax, fe, 2 * n_om, m2, n_om, om, nullptr);
        if (rc != MMA_OK) {
            set_status(rc, "spectrum failed");
            goto fail;
        }
    }
    CK(cudaDeviceSynchronize());
    series.resize(6 * S1);
    CK(cudaMemcpy(series.data(), d_out, sizeof(double) * 6 * S1, cudaMemcpyDeviceToHost));
    {
        // host arrays with the reference's lengths (Nt+2 = n_out+1 for series)
        double** dst[6] = {&out->tgrid, &out->Efield, &out->sourceterm, &out->PopTot, &out->PopInt, &out->expval};
        for (int s = 0; s < 6; s++) {
            *dst[s] = (double*)calloc((size_t)S1, sizeof(double));
            memcpy(*dst[s], series.data() + s * S1, sizeof(double) * S1);
        }
        out->Nt = n_out;
        out->omegagrid = (double*)calloc(n_om, sizeof(double));
        out->FEfield = (double*)calloc(2 * (size_t)n_om, sizeof(double));
        out->Fsourceterm = (double*)calloc(2 * (size_t)n_om, sizeof(double));
        out->FEfieldM2 = (double*)calloc(n_om, sizeof(double));
        out->FsourcetermM2 = (double*)calloc(n_om, sizeof(double));
        CK(cudaMemcpy(out->FEfield, d_spec, sizeof(double) * 2 * n_om, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(out->Fsourceterm, d_spec + 2 * n_om, sizeof(double) * 2 * n_om, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(out->FEfieldM2, d_spec + 4 * n_om, sizeof(double) * n_om, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(out->FsourcetermM2, d_spec + 5 * n_om, sizeof(double) * n_om, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(out->omegagrid, d_spec + 6 * n_om, sizeof(double) * n_om, cudaMemcpyDeviceToHost));
        out->Nomega = n_om;
        if (n_snap > 0) {
            out->psi = (double**)malloc(sizeof(double*) * n_snap);
            for (int s = 0; s < n_snap; s++) {
                out->psi[s] = (double*)calloc(2 * (size_t)n, sizeof(double));
                CK(cudaMemcpy(out->psi[s], d_snap + (size_t)s * 2 * n, sizeof(double) * 2 * n,
                              cudaMemcpyDeviceToHost));
            }
        }
    }
fail:
    cudaFree(d_raw);
    cudaFree(d_fld);
    cudaFree(d_out);
    cudaFree(d_spec);
    cudaFree(d_snap);
    cudaFree(d_scratch);
    cudaFree(d_counter);
    cudaFree(d_inst);
    free_grid(g);
}

// tools.c:423-431
extern "C" void set_time_and_field(inputs_def* in, double* time, double* field, int N)
{
    clear_status();
    if (!in || N < 0 || (N > 0 && (!time || !field))) {
        set_status(MMA_ERR_ARG, "set_time_and_field: bad arguments");
        return;
    }
    in->Efield.tgrid = (double*)calloc((size_t)N, sizeof(double));
    in->Efield.Field = (double*)calloc((size_t)N, sizeof(double));
    for (int i = 0; i < N; i++) {
        in->Efield.tgrid[i] = time[i];
        in->Efield.Field[i] = field[i];
    }
}

// structures.c:92-133
extern "C" output_print_def Set_all_prints(void)
{
    output_print_def r;
    r.Efield = r.FEfield = r.sourceterm = r.Fsourceterm = r.FEfieldM2 = r.FsourceTermM2 = 1;
    r.PopTot = r.tgrid = r.omegagrid = r.PopInt = r.expval_x = 1;
    return r;
}

extern "C" output_print_def Initialise_Printing_struct(void)
{
    output_print_def r;
    memset(&r, 0, sizeof(r));
    return r;
}

// structures.c:15-68
extern "C" void outputs_destructor(outputs_def* o)
{
    if (!o) return;
    double** arrs[11] = {&o->tgrid, &o->omegagrid, &o->Efield, &o->sourceterm, &o->PopTot, &o->FEfield,
                         &o->Fsourceterm, &o->FEfieldM2, &o->FsourcetermM2, &o->PopInt, &o->expval};
    for (auto p : arrs) {
        free(*p);
        *p = nullptr;
    }
}

extern "C" void inputs_destructor(inputs_def* in)
{
    if (!in) return;
    free(in->psi0);
    in->psi0 = nullptr;
    free(in->x);
    in->x = nullptr;
    free(in->Efield.tgrid);
    in->Efield.tgrid = nullptr;
    free(in->Efield.Field);
    in->Efield.Field = nullptr;
}

// tools.c:408-411, structures.c:76-85
extern "C" void free_arr(double* buf) { free(buf); }

extern "C" void free_mtrx(double** buf, int n_rows)
{
    if (!buf) return;
    for (int i = 0; i < n_rows; i++) free(buf[i]);
    free(buf);
}

// ------------------------------------------------------------------------------------------
// Analysis exports of the reference DLL (bound in PythonTDSE.py:80-150): host buffers in,
// malloc'd host results out (freed by free_arr / free_mtrx), computed on the GPU.

// tools.c:206-316 -- the inputs record is passed by value, as in the reference
extern "C" double* window_analysis(inputs_def inputs, double* psi, int num_E, double dE, double Estep, double E_start)
{
    clear_status();
    if (!psi || num_E < 1 || inputs.num_r < 1 || !(inputs.dx > 0.0)) {
        set_status(MMA_ERR_ARG, "window_analysis: invalid arguments");
        return nullptr;
    }
    if (!have_device()) return nullptr;
    const size_t n = (size_t)inputs.num_r + 1;
    int chunk = num_E < 16384 ? num_E : 16384;
    const size_t sb = mma_tdse_pes_scratch_bytes(inputs.num_r, chunk);
    double *d_psi = nullptr, *d_pes = nullptr;
    void* d_sc = nullptr;
    double* out = nullptr;
    int rc;
    CK(cudaMalloc(&d_psi, sizeof(double) * 2 * n));
    CK(cudaMalloc(&d_pes, sizeof(double) * num_E));
    CK(cudaMalloc(&d_sc, sb));
    CK(cudaMemcpy(d_psi, psi, sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    rc = mma_tdse_pes(d_psi, inputs.num_r, inputs.dx, inputs.trg.a, num_E, dE, Estep, E_start, d_pes, d_sc, sb,
                      nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "mma_tdse_pes failed (status %d)", rc);
        goto fail;
    }
    out = static_cast<double*>(malloc(sizeof(double) * num_E));
    CK(cudaMemcpy(out, d_pes, sizeof(double) * num_E, cudaMemcpyDeviceToHost));
    cudaFree(d_psi);
    cudaFree(d_pes);
    cudaFree(d_sc);
    return out;
fail:
    free(out);
    if (d_psi) cudaFree(d_psi);
    if (d_pes) cudaFree(d_pes);
    if (d_sc) cudaFree(d_sc);
    return nullptr;
}

// tools_fftw3.c:158-213 -- rows [N_G][N_freq]
extern "C" double** GaborTransform(double* signal, double dt, int N, int N_freq, int N_G, double t_min, double t_max,
                                   double a)
{
    clear_status();
    if (!signal || N < 2 || N_freq < 1 || N_freq > N / 2 + 1 || N_G < 1) {
        set_status(MMA_ERR_ARG, "GaborTransform: invalid arguments");
        return nullptr;
    }
    if (!have_device()) return nullptr;
    const size_t sb = mma_gabor_scratch_bytes(1, N, N_G);
    double *d_sig = nullptr, *d_g = nullptr;
    void* d_sc = nullptr;
    double** rows = nullptr;
    double* h = nullptr;
    int rc;
    CK(cudaMalloc(&d_sig, sizeof(double) * N));
    CK(cudaMalloc(&d_g, sizeof(double) * (size_t)N_G * N_freq));
    CK(cudaMalloc(&d_sc, sb));
    CK(cudaMemcpy(d_sig, signal, sizeof(double) * N, cudaMemcpyHostToDevice));
    rc = mma_gabor(d_sig, N, 1, dt, N, N_freq, N_G, t_min, t_max, a, d_g, d_sc, sb, nullptr);
    if (rc != MMA_OK) {
        set_status(rc, "mma_gabor failed (status %d)", rc);
        goto fail;
    }
    h = static_cast<double*>(malloc(sizeof(double) * (size_t)N_G * N_freq));
    CK(cudaMemcpy(h, d_g, sizeof(double) * (size_t)N_G * N_freq, cudaMemcpyDeviceToHost));
    rows = static_cast<double**>(malloc(sizeof(double*) * N_G));
    for (int i = 0; i < N_G; i++) {
        rows[i] = static_cast<double*>(malloc(sizeof(double) * N_freq));
        memcpy(rows[i], h + (size_t)i * N_freq, sizeof(double) * N_freq);
    }
    free(h);
    cudaFree(d_sig);
    cudaFree(d_g);
    cudaFree(d_sc);
    return rows;
fail:
    free(h);
    if (d_sig) cudaFree(d_sig);
    if (d_g) cudaFree(d_g);
    if (d_sc) cudaFree(d_sc);
    return nullptr;
}
