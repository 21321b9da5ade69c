// Internal declarations shared by the CUDA kernels and the host driver.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include <complex>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "hosnwt.h"

namespace hos {

// Programmatic dependent launch: kernels are launched with programmatic
// stream serialization.  Every kernel waits for its predecessor's
// completion and memory before it touches data the predecessor may write
// (griddepcontrol.wait is a no-op without a programmatic predecessor), then
// lets its own successor launch, so that the successor's launch and its
// work on constant data (twiddle tables, indices) overlap this kernel.
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Runs a set-up action once per device (thread-safe).  Kernel attributes
// such as the dynamic shared-memory limit belong to a device, so a process
// that drives two GPUs sets them on each; host threads making their first
// launch at the same time are serialised by the mutex.
struct PerDeviceOnce {
  std::mutex m;
  unsigned long long done[4] = {0, 0, 0, 0};  // one bit per device ordinal < 256
  template <typename F>
  void run(F&& f) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    std::lock_guard<std::mutex> g(m);
    if (dev < 0 || dev >= 256) {
      f();
      return;
    }
    unsigned long long& w = done[dev >> 6];
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(w & bit)) {
      f();
      w |= bit;
    }
  }
};

// Set while a graph is captured whose kernels must be fully serialised
// (a body graph that does not accept programmatic dependencies).
extern thread_local bool g_launch_no_pdl;

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = g_launch_no_pdl ? 0 : 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// The same with a thread-block cluster of `cluster` CTAs along x.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_cluster(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                      int cluster, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = cluster;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  cfg.attrs = g_launch_no_pdl ? attr + 1 : attr;
  cfg.numAttrs = g_launch_no_pdl ? 1 : 2;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// ---------------------------------------------------------------------------
// Spectral transforms along one axis.
//
// Every r2r transform of the reference (fourier_FFTW.f90) is separable, so a
// 2-D transform is a pass along x (contiguous) followed by a pass along y.
// One pass computes, for each line and each output k < nout,
//     out[k] = s(k) * gscale * sum_{j in [jlo, min(jhi, nin))} w(j) x[j] cos(pi m(j,k) / (2D))
// with m(j,k) = (aj*j + bj) * (ak*k + bk) + off  (mod 4D).  The six FFTW kinds
// (REDFT00, RODFT00 on the interior, REDFT01, RODFT01, REDFT10, RODFT10) and
// their S2F/F2S normalisations (fourier_FFTW.f90:175-229) are parameter sets
// of this form; sines are cosines shifted by -D.
// ---------------------------------------------------------------------------
enum AxisKind {
  K_C1_S2F = 0,  // REDFT00 * s_2_f (cos, space -> modes)
  K_C1_F2S = 1,  // f_2_s * REDFT00 (cos, modes -> space)
  K_S1_S2F = 2,  // RODFT00 on the interior * s_2_f
  K_S1_F2S = 3,  // f_2_s * RODFT00 on the interior
  K_ZC_S2F = 4,  // REDFT01 / n3_add      (wavemaker z, cos)
  K_ZS_S2F = 5,  // RODFT01 / n3_add      (wavemaker z, sin)
  K_ZC_F2S = 6,  // 0.5 * REDFT10         (wavemaker z, cos)
  K_ZS_F2S = 7,  // 0.5 * RODFT10         (wavemaker z, sin)
};

struct AxisJob {
  const double* in;
  double* out;
  long long in_sk, in_sl;    // stride along the transform axis / between lines
  long long out_sk, out_sl;
  int nlines;
  int N;                     // grid points along the axis
  int nin;                   // inputs j >= nin are zero
  int nout;                  // outputs k < nout are written
  int aj, bj, ak, bk, off;   // angle index m = (aj*j+bj)*(ak*k+bk)+off mod 4D
  int D;                     // table denominator: angle = pi*m/(2D)
  int jlo, jhi;              // summation range [jlo, jhi)
  int klo, khi;              // outputs outside [klo, khi) are zero
  double w0, wm, wl;         // weights for j == 0, interior j, j == N-1
  double s0, sm, sl;         // scales for k == 0, interior k, k == N-1
  double gscale;
  const double* win;         // optional input weights (first pass only): input j
  long long win_sl;          //   of line l is multiplied by win[j * win_sk + l * win_sl]
  long long win_sk;
  const double* q;           // quarter-wave table cos(pi*m/(2D)), m = 0..D
  const double* ty;          // y passes: twiddle rows [j * ldy + k], k <= D/2 (or null)
  int ldy;
  int epi;                   // 1: the batch's AccEpi follows each output write
  // work decomposition of the x pass (set by the launcher)
  int mode;                  // 0 direct, 1 output symmetry k <-> D-k, 2 input symmetry j <-> D-j
  int nlane;                 // lane outputs: tiles of 32 cover [0, nlane)
  int ntile;
  int nchunk, chunk;         // the sum is split over nchunk CTAs of `chunk` terms
  int ta, tb;                // term range [ta, tb) (interior terms or symmetric pairs)
  double* part;              // nlines * ntile * nchunk * 64 partial sums (nchunk > 1)
  unsigned int* cnt;         // nlines * ntile arrival counters (nchunk > 1)
  // two-level passes (REDFT00 / RODFT00 kinds with D = A * B)
  int A, B;                  // 0 when the direct sum is used
  double* cs;                // nlines * B * (A + 1) * 2 partial cos/sin sums
};

constexpr int kMaxJobs = 16;

// HOS order accumulation (HOSphis_modes, resol_HOS.f90:716-764) fused into
// the final pass of the transform that produces its first term z1 =
// phizi(iHOS, 1): at every output element e,
//   phimext[e] = -sum_{j=iHOS..2} z_j[e] eta_{j-1}[e] - z1 eta_0[e]
//   phizm[e]   =  sum_{j=iHOS..2} z_j[e] eta_{j-2}[e] + z1
// in the order of k_hos_accum.  z[j-1] = phizi(iHOS+1-j, j), e[j-1] = eta^j/j!.
constexpr int kAccMax = 8;
struct AccEpi {
  int iHOS;
  const double* z[kAccMax];
  const double* e[kAccMax];
  double* phimext;
  double* phizm;
};
#if defined(__CUDACC__)
__device__ __forceinline__ void acc_epilogue(const AccEpi& a, long long i, double z1) {
  double pm = 0.0, pz = 0.0;
  for (int j = a.iHOS; j >= 2; --j) {
    const double z = __ldcg(a.z[j - 1] + i);
    pm = pm - z * __ldcg(a.e[j - 1] + i);
    pz = pz + z * __ldcg(a.e[j - 2] + i);
  }
  a.phimext[i] = pm - z1 * __ldcg(a.e[0] + i);
  a.phizm[i] = pz + z1;
}
#endif

// A batch of jobs for one launch.  Kernels take the batch by value as their
// parameters, whose size costs launch time, so a launch passes the smallest
// capacity NJ (1, 2, 4, 8 or kMaxJobs) that holds its jobs.
template <int NJ>
struct AxisBatchT {
  AxisJob job[NJ];
  int start[NJ + 1];         // first CTA of each job
  int njobs;
  int early;                 // 1: the twiddle tables are constant and are staged
                             //    before waiting for the previous kernel
  AccEpi acc;                // applied to the outputs of jobs with epi set
};
using AxisBatch = AxisBatchT<kMaxJobs>;

// grid ids of the transform requests
enum GridId { GRID_N = 0, GRID_BIG = 1, GRID_ADD = 2 };

// One (possibly 2-D) transform request on device memory.
struct XfReq {
  int grid;                  // GridId
  int dir;                   // +1 S2F, -1 F2S
  int csx, csy;              // 0 cos, 1 sin
  const double* in;
  int in_ld, nin1, nin2;     // input leading dim and nonzero extent
  double* out;
  int out_ld, nout1, nout2;  // output leading dim and written extent
  double scale;
  const double* win = nullptr;  // optional weights: input (i1, i2) times win[i1 + win_ld * i2]
  int win_ld = 0;
  const AccEpi* acc = nullptr;  // optional accumulation on the outputs (final pass)
};

struct Tables;

// Launch the x passes (and y passes when n2 > 1) of up to kMaxJobs requests.
// tmp[i] holds the x-pass result of request i when a y pass follows.
void launch_transforms(const XfReq* reqs, int nreq, const Tables& tb, double* const* tmp,
                       cudaStream_t st);

struct Tables;
// F2S along y only (FOURIER_2_SPACE_y, fourier_FFTW.f90:340-428) of nlines
// lines that are contiguous in memory; cs: 0 cos, 1 sin.
void launch_y_f2s(const Tables& tb, const double* in, int nlines, long long y_stride, double* out,
                  long long out_y_stride, int cs, cudaStream_t st);

// ---------------------------------------------------------------------------
// FFT-based passes (fft.cu).  A REDFT00 / RODFT00 pass of length N = D + 1
// over many lines runs as one real DFT of length D per line (two lines
// packed into one complex DFT), computed by Stockham stages in shared
// memory; a prime D goes through Rader's cyclic convolution of length D - 1.
// ---------------------------------------------------------------------------
constexpr int kFftMaxSt = 16;      // stages of one complex FFT
constexpr int kFftMaxRadix = 127;  // largest odd prime factor of a stage

// Division by a constant d as multiply-high (Granlund and Montgomery, 1994):
// with s = ceil(log2 d) and m = floor(2^32 (2^s - d) / d) + 1,
// x / d = (mulhi(x, m) + x) >> s for every 32-bit x.  The constants of
// the FFT stage loops are set on the host with the plans.
struct FastDivC {
  unsigned d, m, s;
};
inline FastDivC make_fastdiv(unsigned d) {
  unsigned s = 0;
  while ((1ULL << s) < d) ++s;
  const unsigned long long m = ((1ULL << 32) * ((1ULL << s) - d)) / d + 1ULL;
  return FastDivC{d, (unsigned)m, s};
}

struct FftStages {
  int L;                     // complex length
  int nst;                   // number of Stockham stages
  int rad[kFftMaxSt];        // radix of each stage, in order
  int twoff[kFftMaxSt];      // offset of each stage's twiddles in stw
  // division constants of stage s: L / R, Ns, and for an odd radix given at
  // run time (R + 1) / 2 - 1 and (R + 1) / 2
  FastDivC dnb[kFftMaxSt], dns[kFftMaxSt], dh1[kFftMaxSt], dh[kFftMaxSt];
  const double2* tw;         // exp(-2 pi i q / L), q = 0..L-1
  const double2* stw;        // stage twiddles: stage s (radix R, Ns the product of the
                             //   earlier radices) holds exp(-2 pi i t k / (Ns R)) at
                             //   twoff[s] + (t - 1) Ns + k, t = 1..R-1, k < Ns
};

// In-place mixed-radix FFT of length L (radices 2, 3, 4, 5, 7, 8): the
// decimation-in-frequency form takes natural order to digit-reversed order,
// the decimation-in-time form digit-reversed order back to natural order.
// Stage s has span S (L over the product of the earlier radices) and
// m = S / R; its twiddles exp(-2 pi i q j / S) sit at off[s] + (q - 1) m + j.
struct FftInplace {
  int L;
  int nst;
  int rad[kFftMaxSt];
  int off[kFftMaxSt];
  FastDivC dnb[kFftMaxSt], dm[kFftMaxSt];  // division constants: L / R and m of stage s
  const double2* tw;
};

enum FftMode { FFT_STOCKHAM = 0, FFT_RADER = 1, FFT_BLUESTEIN = 2 };

// Device description of one transform length D (built once per context).
struct FftDesc {
  int D;
  int mode;                  // FftMode
  FftStages fft;             // Stockham FFT of length D (mode 0) or D - 1 (mode 1)
  const int* gperm;          // rader: input index g^m mod D, m = 0..D-2
  const int* gscat;          // rader: output index g^-n mod D, n = 0..D-2
  const double2* bconj;      // rader: conj(FFT(exp(-2 pi i g^-q / D))) / (D - 1)
  FftInplace ip;             // bluestein: in-place FFT of the convolution length M
  const double2* chirp;      // bluestein: exp(-i pi j^2 / D), j < D
  const double2* hrev;       // bluestein: conj(FFT_M(chirp kernel)) / M, digit-reversed
  const double2* trig;       // (cos, 2 sin)(pi j / D), j = 0..D
};

struct FftPlanInfo {
  int D = 0;
  int mode = 0;
  int M = 0;                 // bluestein convolution length (FP64 tables)
  int M_df = 0;              // the same for the double-float tables
  const FftDesc* dev = nullptr;     // FP64 tables
  const FftDesc* dev_df = nullptr;  // double-float tables of the same plan
  double cost_line = 0.0;    // FP64 instructions per line (two lines share one complex FFT)
  double cost_line_df = 0.0; // the same in FP64-instruction time with a double-float DFT
};

// Build the device tables of length D; device allocations are appended to
// `allocs` (freed by the owner).  The cheapest of a Stockham FFT of length D
// (prime factors up to kFftMaxRadix), Rader's algorithm (D prime) and
// Bluestein's chirp convolution is taken.  Returns false on an allocation
// failure or a length whose convolution does not fit in shared memory.
bool build_fft_plan(int D, std::vector<void*>& allocs, FftPlanInfo* out);

struct AxisJob;
// FP64 instructions per line of the FFT pass of job J with plan f.
double fft_line_cost(const FftPlanInfo& f);

struct Tables {
  int n1, n2, nd1, nd2, n3_add;
  int nsm;                   // SMs of the device (sizes the split of the sums)
  double* part;              // scratch for partial sums of split transforms
  long long part_cap;        // capacity (doubles)
  unsigned int* cnt;         // arrival counters (zero between launches)
  int cnt_cap;
  double* cs;                // scratch of the two-level passes (may be null)
  long long cs_cap;
  bool q_const = true;       // tables written before the first launch that reads them
  // twiddle rows of the y passes (cos, sin kinds) for D = n2-1 and nd2-1
  const double* ty_n2[2] = {nullptr, nullptr};
  const double* ty_nd2[2] = {nullptr, nullptr};
  int ldy_n2 = 0, ldy_nd2 = 0;
  // quarter-wave tables for D = n1-1, n2-1, nd1-1, nd2-1, n3_add
  const double* q_n1;
  const double* q_n2;
  const double* q_nd1;
  const double* q_nd2;
  const double* q_add;
  // FFT plans of the axis lengths (x and y, free-surface and dealiased grids)
  FftPlanInfo fft[4];
  int nfft = 0;
};

// The plan of tb for J's length when the FFT pass should run J (a REDFT00 /
// RODFT00 job over enough lines to fill the GPU, whose FFT costs fewer FP64
// instructions per line than `cost_other`), else null.  The environment
// variable HOSNWT_FFT=0 turns the FFT passes off and HOSNWT_FFT=1 takes
// them whenever a plan exists (read once when the library loads).
const FftPlanInfo* fft_choice(const AxisJob& J, const Tables& tb, double cost_other);
// Launch the FFT passes of b's jobs, job i with plan[i].
void launch_fft_jobs(const AxisBatch& b, const FftPlanInfo* const* plan, const Tables& tb, cudaStream_t st);
// Layout tuning of the FFT passes: with recording on (this thread), launches
// whose batch has no tuned layout are recorded; fft_tune_run times the
// layouts of the recorded batches on `st` (outside any capture) and keeps
// the fastest.  Returns the number of batches tuned, -1 on a CUDA error.
bool fft_tune_enabled();
void fft_tune_record(bool on);
int fft_tune_run(cudaStream_t st);

// FP64 FMAs of the transform passes launched from this host thread since
// the counter was last reset (the algorithm's own count: terms times
// outputs, as the launch helpers pick them).  The host reads it around the
// capture of a step graph.
extern thread_local double g_xform_fmas;

// With HOSNWT_FUSED_PASS=1 in the environment (read once when the library
// loads), x passes of few lines (2-D tanks) run both two-level passes in one
// kernel (two_level_fused) instead of two launches.  Off by default: on
// GB300 the single transform is faster but a whole 2-D step is not, and an
// ensemble of tanks is slower (the fused CTAs repeat table staging and
// pass 1).
extern const bool g_fused_enabled;

// FP64 FMA throughput of the current device in GFLOP/s.
double measure_fp64_peak_gflops();

// Build the quarter-wave table cos(pi*m/(2D)), m = 0..D, on the host.
std::vector<double> quarter_table(int D);
// Twiddle rows of a REDFT00 (sin_kind false) or RODFT00 y pass of length N:
// row j holds cos(pi (2 j k + off) / (2D)) for k = 0..D/2 (off = 0 or 3D),
// the same values as the quarter-wave table gives; *ld is the row length.
std::vector<double> y_twiddle_rows(int N, bool sin_kind, int* ld);

}  // namespace hos
