// The tank context: parameters, host tables and device buffers.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <vector>

#include "hosnwt.h"
#include "hosnwt_internal.h"

namespace hos {

// Device scalar slots (one double array on the device).
enum Scalar {
  SC_T0 = 0,       // t_o of the RK step
  SC_H = 1,        // h_loc
  SC_TIME = 2,     // time of the current stage
  SC_DT = 3,       // h_loc * c_s of the current stage
  SC_ALPHA = 4,    // ramp alpha, alphat, alphatt of the last wavemaker law
  SC_ALPHAT = 5,   // evaluation (the reference's globals)
  SC_ALPHATT = 6,
  SC_POSTOP = 7,   // pos1st(n3, 1) of the last evaluation
  SC_ERR = 8,      // embedded error of the last step
  SC_PHIS0 = 9,    // phisrk0 (mean mode of phis)
  SC_COUNT = 16
};

// Offsets of the 10 RK arrays inside one state vector (runge_kutta.f90:81-93).
struct StateLayout {
  long long off[10];
  long long size;
};
enum StateIdx { S_G1 = 0, S_G2, S_AADD1, S_AADD2, S_AADDR, S_AADD3, S_A1ST, S_ETA1ST, S_A2ND, S_ETA2ND };

struct Params {
  // numerics
  int n1, n2, n3, n3a, nd1, nd2, M, p1, p2, l_add;
  // case
  int icase, igeom, iramp, iabsnb, i_wmk, ibat;
  // nondimensional
  double h, Tscale, xlen, ylen, xlen_add, d_hinge, Tramp, T_stop, f_out;
  double nu_mono, w_mono, T_mono, amp_mono, theta_mono, ph_mono, aslosh;
  int islosh;
  double toler, dt_stab, delt, delt_out;
  double delx, dely, delz;
};

struct Dev {
  // tables
  double *omega = nullptr, *kx = nullptr, *ky = nullptr, *kth_ext = nullptr, *kth1 = nullptr;
  double *nu = nullptr, *k_add_thk = nullptr, *kx_add = nullptr, *cosk = nullptr, *sink = nullptr;
  double *csh = nullptr, *ksh = nullptr, *kycsh = nullptr, *kxcsh = nullptr;  // [i1 + n1*i3 + n1*n3a*j2]
  double *ext = nullptr;        // (n3a - n3) x 4 extension weights
  double *pos_re = nullptr, *pos_im = nullptr;  // pos_ini (n2 x nf)
  double *freq_w = nullptr, *gzed = nullptr;
  double *eiwt = nullptr;       // 2*nf scratch: cos/sin(w t)
  double *mat_coscos = nullptr;
  double *q_n1 = nullptr, *q_n2 = nullptr, *q_nd1 = nullptr, *q_nd2 = nullptr, *q_add = nullptr;
  // RK state
  double *y0 = nullptr, *ys = nullptr, *k[5] = {}, *ynew = nullptr;
  double *eta = nullptr, *phis = nullptr, *deta = nullptr;
  double *eta_c = nullptr, *phis_c = nullptr, *deta_c = nullptr;
  // RHS workspace, free-surface grid
  double *etam = nullptr, *phim = nullptr, *eta_sp = nullptr;
  double *w_eta_x = nullptr, *w_eta_y = nullptr, *w_phi_x = nullptr, *w_phi_y = nullptr;
  double *phix_add = nullptr, *phiy_add = nullptr, *phiz_add = nullptr, *phit_add = nullptr;
  double *phi_add = nullptr, *diag = nullptr;
  double *phit_add1 = nullptr, *phiz_add1 = nullptr, *a1k = nullptr, *phiz1st = nullptr, *rhs1 = nullptr;
  double *pmode[3] = {};        // S2F of phix/phiy/phiz_add
  double *X1 = nullptr, *X2 = nullptr, *X3 = nullptr, *det = nullptr, *dph = nullptr;
  double *NL1 = nullptr, *NL2 = nullptr;
  // big grid
  std::vector<double*> etapm, phizm, aHOS;
  std::vector<double*> phizi;   // (m, j) packed
  double *etax = nullptr, *etay = nullptr, *phisx = nullptr, *phisy = nullptr, *gradeta2 = nullptr;
  double *phimext = nullptr, *phizMm1 = nullptr, *tbig = nullptr, *tbig2 = nullptr;
  double *pxe = nullptr, *pye = nullptr, *pze = nullptr, *A1 = nullptr, *A3 = nullptr;
  double *t1 = nullptr, *geta2phiz = nullptr, *geta2phiz2 = nullptr;
  double* grp[24] = {};         // dealiasing groups of the quadratic terms
  // wavemaker grid
  double *bc1 = nullptr, *bcr = nullptr;
  // second-order wavemaker (i_wmk = 2)
  double *kx2cshx = nullptr, *kycshx = nullptr, *kshx = nullptr;  // [i1 + n1 (i2 + n2 i3)], i3 < n3
  double *k_add = nullptr;                                         // n3_add x n2
  double *dnux = nullptr, *dgzed = nullptr, *dposdy_re = nullptr, *dposdy_im = nullptr;
  static constexpr int kW2 = 120;
  double* w2[kW2] = {};  // work fields of the second order, max(n1 n2, n3_add n2) each
  // 3-D phiadd_SL workspace (n1 * n3a * n2 each)
  double *Q[5] = {}, *B[5] = {};
  // transform temporaries
  double *xtmp[kMaxJobs] = {};
  double *xtmp2[kMaxJobs] = {};  // temporaries of the wavemaker branch
  double *xtmp3[kMaxJobs] = {};  // temporaries of the eta-power branch
  static constexpr int kDealiasTmp = 8;
  double *dtmp[kDealiasTmp] = {};  // truncated modes of batched dealiasing (main stream)
  double *ptmp = nullptr;          // truncated modes of the eta-power dealiasing
  // scalars and reductions
  double *sc = nullptr;
  double *part = nullptr;       // partial sums / maxima
  unsigned int *counter = nullptr;
  double *probe_out = nullptr;
  double *host_sc = nullptr;    // pinned mirror of the scalar slots
  double *host_io = nullptr;    // pinned staging of hosnwt_runge4_adapt2's arrays
};

// Step control of HOS-NWT.f90:498-571 on the device: one output interval
// runs as a CUDA-graph WHILE loop whose body is one RK4(5) step, the
// accept/reject decision and the accept.  The block is copied in before
// the loop and out after it.
struct StepCtl {
  double time_cur, h_rk, time_next, err;
  int n_acc, n_rej;
  int endramp;               // the reference's endramp flag
  int accept;                // 1: the step just taken is accepted
  int end_ramp_now;          // 1: this accept removes a_add_ramp from a_add_1
  int status;                // 0 ok, 1 non-finite error estimate, 2 step limit
  int iters;                 // attempted steps
  int pad;
};
struct CtlParams {
  double toler, dt_stab, delt_out, Tramp;
  int iramp;
  int max_iters;
  cudaGraphConditionalHandle cond;
};

struct Ctx {
  hosnwt_input in{};
  hosnwt_numerics num{};
  Params P{};
  std::string err;
  // host tables kept for the oracle-free host logic
  std::vector<double> kx, ky, cx, cy, cz, omega;
  std::vector<std::complex<double>> pos_ini;  // n2 x nf, i2 fastest
  std::vector<std::complex<double>> dposdy_ini;  // d pos_ini / dy, n2 x nf
  std::vector<double> freq_w, gzed;
  std::vector<double> probes;  // nondimensional (x, y)
  int nprobes = 0;
  int nf = 0;
  double k_mono = 0.0;  // wave number of the first wave component (initial_condition.f90:175, 209-210)
  StateLayout L{};
  Dev d{};
  Tables tb{};
  Tables tb2{};                   // transform scratch of the wavemaker branch
  Tables tb3{};                   // transform scratch of the eta-power branch
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;     // wavemaker branch of each right-hand side
  cudaStream_t st3 = nullptr;     // eta powers and |grad eta|^2 with their dealiasing
  cudaEvent_t ev_fork = nullptr, ev_eta = nullptr, ev_join = nullptr, ev_pow = nullptr;
  cudaEvent_t ev_acc = nullptr, ev_dl = nullptr;  // intermediate-order dealiasing
  static constexpr int kPowEvents = 8;
  cudaEvent_t ev_pw[kPowEvents] = {};  // eta powers final up to a given order
  cudaGraphExec_t step_graph = nullptr;
  cudaGraphExec_t loop_graph = nullptr;  // device-controlled output interval (built on first use)
  int loop_state = 0;                     // 0 not tried, 1 built, -1 unavailable (host loop)
  bool loop_pdl = false;                  // the loop body keeps programmatic launches
  StepCtl* ctl_dev = nullptr;
  StepCtl* ctl_host = nullptr;            // pinned
  double time_cur = 0.0;
  int endramp = 0;
  long long n_rhs = 0;
  int kernels_per_step = 0;
  double fmas_per_step = 0.0;     // FP64 FMAs of the transforms in one step graph
  double dev_ms = 0.0;            // device time of steps and accepts (CUDA events)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int nparts = 0;
  std::vector<void*> allocs;
};

// host setup (host.cpp)
int setup(Ctx& c, const char* wave_dir, const double* probes_xy, int nprobes);

// device pipeline (rhs.cu)
int alloc_device(Ctx& c);
void free_device(Ctx& c);
void enqueue_rhs(Ctx& c, const double* y, double* k, bool rk_mode, cudaStream_t st);
void enqueue_step(Ctx& c, cudaStream_t st);
void enqueue_initialize(Ctx& c, cudaStream_t st);
void enqueue_probes(Ctx& c, cudaStream_t st);
void enqueue_diagnostics(Ctx& c, double* out, cudaStream_t st);
void enqueue_slope_filter(Ctx& c, int dir, cudaStream_t st);
void enqueue_accept(Ctx& c, bool end_ramp, cudaStream_t st);
// Body of the device-controlled loop: set t_o and h_loc from the control
// block, one RK4(5) step, the accept/reject decision (sets the loop
// condition), the accept.
void enqueue_ctl_step(Ctx& c, StepCtl* ctl, const CtlParams& p, cudaStream_t st);
void enqueue_set_scalar(Ctx& c, int slot, double v, cudaStream_t st);

}  // namespace hos
