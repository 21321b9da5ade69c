/*
 * hosnwt.h -- C ABI of the GB300-native HOS numerical wave tank.
 *
 * The library (libhosnwt.so) replaces the FP64 hot path of LHEEA/HOS-NWT:
 * one adaptive RK4(5) step (runge_kutta.f90:81-360) with its five nonlinear
 * right-hand sides (resol_HOS.f90:270-656), the spectral transforms
 * (fourier_FFTW.f90:89-653), the wavemaker additional potential
 * (resol_wmkr.f90:109-210, 1124-1187) and the absorbing zone.  Around it sits a
 * host driver that keeps the reference's inputs (input_HOS-NWT.dat, prob.inp,
 * .cfg/.dat wave files), its step control (HOS-NWT.f90:498-571) and its probe
 * output.
 *
 * Conventions: every function returns 0 on success or a HOSNWT_ERR_* code
 * (never aborts); hosnwt_last_error() gives the message.  Host arrays are
 * column-major with i1 fastest (Fortran layout of the reference), sizes
 * (n1,n2) for free-surface fields and (n3_add,n2) for wavemaker modes,
 * n3_add = 2*(n3-1).  Pointers are borrowed for the duration of the call.
 * A context is not thread-safe; independent contexts are.
 */
#ifndef HOSNWT_H
#define HOSNWT_H

#ifdef __cplusplus
extern "C" {
#endif

#define HOSNWT_OK 0
#define HOSNWT_ERR_ARG 1
#define HOSNWT_ERR_CUDA 2
#define HOSNWT_ERR_NAN 3
#define HOSNWT_ERR_TIMEOUT 4
#define HOSNWT_ERR_DT_UNDERFLOW 5
#define HOSNWT_ERR_IO 6
#define HOSNWT_ERR_UNSUPPORTED 7

/* Physical/case parameters: the fields of input_HOS-NWT.dat in file order
 * (read_input, input.f90:62-201), dimensional as in the file. */
typedef struct hosnwt_input {
  double xlen, ylen, h;
  int icase;
  int islosh;
  double aslosh;
  double amp_mono, nu_mono, theta_mono, ph_mono;
  int ibat;
  double xd_mono;
  char file_name[256];
  int i_cut;
  double nuc_low, nuc_high;
  double Hs, Tp, gamma;
  int iseed;
  int i_wmk, igeom;
  double d_hinge;
  int iramp;
  double Tramp;
  int iabsnb;
  double xabsf, coeffabsf;
  int iprobes;
  char pro_file[256];
  double T_stop, toler, f_out;
  int idim, i3d, imodes, iwmk, i_sw;
} hosnwt_input;

/* Numerical sizes: compile-time parameters of the reference
 * (common_vars.f90:31-43), runtime here. */
typedef struct hosnwt_numerics {
  int n1, n2, n3, mHOS, p1, p2;
} hosnwt_numerics;

/* Derived quantities of a context (HOS-NWT.f90:99-244). */
typedef struct hosnwt_info {
  int n1, n2, n3, n3_add, nd1, nd2, mHOS, p1, p2;
  double Tscale, xlen, ylen, dt_stab, delt, delt_out, T_stop, toler;
  double time_cur;
  int nprobes;
  long long n_rhs;         /* right-hand sides evaluated so far */
  int kernels_per_step;    /* kernel launches in one RK4(5) step graph */
  double device_ms;        /* device time of all steps and accepts so far
                              (CUDA events on the context's stream) */
  double fmas_per_step;    /* FP64 FMAs of the transform passes in one step
                              graph (terms x outputs of the algorithm run) */
  int step_control;        /* where hosnwt_advance decides accept/reject
                              (HOS-NWT.f90:498-571): 0 not yet chosen (no
                              advance so far), 1 the host, once per step;
                              2 the device, a CUDA-graph loop per output
                              interval with programmatic launches; 3 the
                              device, kernels fully serialised in the loop */
} hosnwt_info;

typedef struct hosnwt_ctx hosnwt_ctx;

/* read_input (input.f90:62-201): parse input_HOS-NWT.dat. */
int hosnwt_read_input(const char* path, hosnwt_input* out);

/* Set up a tank on the current CUDA device: initiate_parameters,
 * nondimensionalisation, time-step choice, meshes, wave synthesis, absorbing
 * zone, spectral tables and the initial condition (HOS-NWT.f90:86-432,
 * initial_condition.f90:32-482).  wave_dir is the directory of the
 * .cfg/.dat files (icase 3); probes_xy holds nprobes (x, y) positions in
 * metres (prob.inp, output.f90:108-141), or NULL. */
int hosnwt_create(const hosnwt_input* in, const hosnwt_numerics* num,
                  const char* wave_dir, const double* probes_xy, int nprobes,
                  hosnwt_ctx** out);
void hosnwt_destroy(hosnwt_ctx* ctx);
const char* hosnwt_last_error(const hosnwt_ctx* ctx);
int hosnwt_get_info(const hosnwt_ctx* ctx, hosnwt_info* info);

/* runge4_adapt2 (runge_kutta.f90:81-360): one RK4(5) step of size h_loc from
 * time t_o on HOST arrays (eta, phis, eta1st, eta2nd, a1st, a2nd: n1 x n2;
 * a_add_*: n3_add x n2), updated in place; err receives the embedded error
 * estimate.  Same argument order and meaning as the Fortran routine. */
int hosnwt_runge4_adapt2(hosnwt_ctx* ctx, double t_o, double* eta, double* phis,
                         double* a_add_rk_1, double* a_add_rk_2, double* a_add_rkramp,
                         double* a_add_rk_3, double* eta1st, double* eta2nd,
                         double* a1st, double* a2nd, double h_loc, double* err);

/* Device-resident variant: one RK step of size h_loc from the context's
 * current time on the device state.  The result is kept as a candidate;
 * hosnwt_accept() makes it the state (HOS-NWT.f90:531-560). */
int hosnwt_step(hosnwt_ctx* ctx, double h_loc, double* err);
int hosnwt_accept(hosnwt_ctx* ctx, double h_loc);

/* Inner adaptive loop of HOS-NWT.f90:498-571 up to time_next (nondimensional)
 * with step control on the host; h_rk is the in/out step size. */
int hosnwt_advance(hosnwt_ctx* ctx, double time_next, double* h_rk, int* n_acc, int* n_rej);

/* Whole time loop (HOS-NWT.f90:446-581) writing Results/probes.dat,
 * Results/vol_energy.dat and, when i3d = 1, Results/3d.dat into results_dir
 * (NULL: no files), in the formats of output.f90 (input echo, 61d13.5 probe
 * records, 5(ES12.5,X) energies, free-surface zones with tecplot = 11), with
 * check_slope after each output interval. */
int hosnwt_run(hosnwt_ctx* ctx, const char* results_dir);

/* Diagnostics of the current state (vol_energy.f90:36-119 and
 * check_slope's slopes): out[0] volume, out[1] potential and out[2] kinetic
 * energy (phis + phi_add of the last right-hand side times deta), out[3] and
 * out[4] max |eta_x| and max |eta_y| of the last right-hand side. */
int hosnwt_diagnostics(hosnwt_ctx* ctx, double* out5);
/* check_slope (initial_condition.f90:687-716): filter eta and phis (cut at
 * 0.7 of the modes) in each direction whose slope exceeds 8; *filtered gets
 * bit 0 (x) and bit 1 (y) of what was filtered. */
int hosnwt_check_slope(hosnwt_ctx* ctx, int* filtered);

/* Copy the physical state to host arrays (n1 x n2 each; NULL to skip). */
int hosnwt_get_state(hosnwt_ctx* ctx, double* eta, double* phis, double* deta);
/* Copy the 10 arrays runge4_adapt2 advances (same order and shapes) from
 * the device state (the reference's eta, phis, a1st_add, a2nd_add,
 * a_add_ramp, a3rd_add, eta1st, eta2nd, a1st, a2nd). */
int hosnwt_get_rk_state(hosnwt_ctx* ctx, double* eta, double* phis, double* a_add_1,
                        double* a_add_2, double* a_add_ramp, double* a_add_3, double* eta1st,
                        double* eta2nd, double* a1st, double* a2nd);
/* Replace eta and phis (physical space, n1 x n2) on the device. */
int hosnwt_set_state(hosnwt_ctx* ctx, const double* eta, const double* phis);

/* Probe elevations at the context's probes (output.f90:265-282),
 * nondimensional; out holds nprobes values. */
int hosnwt_probes(hosnwt_ctx* ctx, double* out);

/* Test hook: solveHOS2 (resol_HOS.f90:270-656) on host arrays.  y and k hold
 * the 10 RK state arrays in runge4_adapt2's order: G1, G2, a_add_1, a_add_2,
 * a_add_ramp, a_add_3, a1st, eta1st, a2nd, eta2nd.  `alpha_prev` and
 * `pos_top_prev` are the wavemaker ramp and paddle top position of the
 * previous stage (the reference's volume correction reads them). */
int hosnwt_solveHOS2(hosnwt_ctx* ctx, const double* const* y, double* const* k,
                     double delta_t, double time, double alpha_prev, double pos_top_prev);

/* Snapshot hook for training a surrogate of the high HOS orders: the
 * fields of the last right-hand side evaluated on this context (stage 5 of
 * the last hosnwt_step, or the last hosnwt_solveHOS2), on the dealiased
 * grid nd1 x nd2, column-major: eta_big = eta (etapm(:,:,1)) and phizm =
 * the M vertical-velocity terms phizm(:,:,1..M) of HOSphis_modes
 * (resol_HOS.f90:665-915), order after order (M * nd1 * nd2 doubles), each
 * after its partial dealiasing.  Synchronises the context's stream. */
int hosnwt_hos_terms(hosnwt_ctx* ctx, double* eta_big, double* phizm);

/* Test hook: one spectral transform on host arrays.
 * grid: 0 free surface (n1 x n2), 1 dealiased (nd1 x nd2), 2 wavemaker
 * (n3_add x n2).  dir: +1 SPACE_2_FOURIER, -1 FOURIER_2_SPACE.
 * csx/csy: 0 cos, 1 sin (csx is the z kind on the wavemaker grid).
 * Same results as DCT_FFTW / IDCT_FFTW and their _big/_add variants
 * (fourier_FFTW.f90:235-653). */
int hosnwt_transform(hosnwt_ctx* ctx, int grid, int dir, int csx, int csy,
                     const double* in, double* out);

/* Measurement hooks (no counterpart in the reference).
 * hosnwt_time_transform: average device time (ms, CUDA events on the
 * context's stream) of one batched transform of `batch` requests on the
 * given grid with nonzero input extent nin1 x nin2 and written output
 * extent nout1 x nout2, from `nrep` of them run back to back in one CUDA
 * graph (as the step graph runs its transforms).
 * hosnwt_fp64_peak: FP64 FMA throughput of the current device (GFLOP/s). */
int hosnwt_time_transform(hosnwt_ctx* ctx, int grid, int dir, int csx, int csy, int nin1, int nin2,
                          int nout1, int nout2, int batch, int nrep, double* ms_per_launch);
int hosnwt_fp64_peak(double* gflops);

/* No counterpart in the reference.  A transform for callers that cannot
 * allocate device memory: hosts whose GPU memory is owned by their own pool
 * or a fixed budget reserved at start-up, and time loops that must not let
 * cudaMalloc/cudaFree synchronise the device.  It needs no context and
 * allocates nothing: the caller passes device arrays `in` and `out` of
 * `nlines` lines of n doubles each (line stride n); the result equals
 * hosnwt_transform on the free-surface grid of a 2-D tank (n2 = 1) with
 * n1 = n: SPACE_2_FOURIER (dir = +1) or FOURIER_2_SPACE (dir = -1), cs 0 cos
 * (REDFT00), 1 sin (RODFT00 on the interior).  Work goes on `stream` (a
 * cudaStream_t; NULL for the legacy default stream).
 * Its only extra memory is one fixed array of about 2.3 MB in the library,
 * held by every GPU that loads it until the process exits; lengths
 * 5 <= n <= HOSNWT_NOALLOC_MAX_N, anything else returns HOSNWT_ERR_ARG.
 * The first call on each device looks up that array's device address; make
 * that first call before any stream capture.  Every call shares the array:
 * calls that overlap on the GPU race and must be serialised by the caller. */
#define HOSNWT_NOALLOC_MAX_N 16385
int hosnwt_transform_noalloc(int dir, int cs, int n, int nlines, const double* in, double* out,
                             void* stream);

/* Batched ensemble (independent tanks, no collective): advance every context
 * to time_next (its own nondimensional clock) with per-tank adaptive dt.
 * Launches of different tanks are interleaved on their own streams. */
int hosnwt_advance_many(hosnwt_ctx* const* ctxs, int n, const double* time_next,
                        double* h_rk);

/* Tensor-core contraction of the surrogate (tc_gemm.cu), on device
 * pointers: D = act(A B^T + bias + Dadd) with A (M x K, row stride lda) and
 * B (N x K, row stride ldb) in BF16, FP32 accumulation, D FP32 (d_bf16 = 0)
 * or BF16 (row stride ldd); bias (N) and Dadd (FP32, M x N, row stride ldd)
 * may be null; act 0 = none, 1 = GELU (tanh form).  K, lda and ldb must be
 * multiples of 8 and A, B 16-byte aligned.  *err (device) is set to 1 if a
 * wait inside the kernel timed out.  Asynchronous on `stream` (a
 * cudaStream_t, null for the default stream). */
int hosnwt_tc_gemm_bf16(const void* A, long long lda, const void* B, long long ldb, void* D, long long ldd,
                        int d_bf16, int M, int N, int K, const float* bias, int act, const float* Dadd,
                        unsigned* err, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HOSNWT_H */
