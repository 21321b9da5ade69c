// A context-free spectral transform that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host code whose device memory is
// owned by its own pool or fixed budget (for instance a coupled solver that
// reserves all of the GPU at start-up), or a time loop that must not let
// cudaMalloc/cudaFree synchronise the device and stall its other streams.
// hosnwt_transform_noalloc serves them: the caller passes device input and
// output arrays, and the only other memory it touches is the fixed array
// below, which every GPU that loads the library holds until the process exits.
//
// The array holds the quarter-wave twiddle table and the partial sums and
// arrival counters of the split transform sums.  It is shared by every call:
// calls that overlap on the GPU (two streams, or two host threads) race on it
// and give wrong results; serialise them.  Each call clears the counters and
// rebuilds the table before its transform.
#include <cuda_runtime.h>

#include <mutex>

#include "hosnwt.h"
#include "hosnwt_internal.h"

namespace hos {
namespace {

// layout of the scratch array (doubles)
constexpr int kNoallocMaxN = HOSNWT_NOALLOC_MAX_N;            // longest transform
constexpr long long kTableLen = kNoallocMaxN + 7;             // cos table, D <= max N - 1
constexpr long long kPartLen = 64LL * 4096;                   // partial sums
constexpr int kCntLen = 4096;                                 // arrival counters
constexpr long long kScratchLen = kTableLen + kPartLen + kCntLen / 2;

static __device__ __align__(256) double g_noalloc_scratch[kScratchLen];
// the regions are disjoint at the largest length: the table holds m = 0..D
static_assert(kTableLen >= kNoallocMaxN, "cos table shorter than the longest transform");

std::mutex g_setup_mutex;
double* g_scratch_addr[256] = {};  // device address of the array, per device

// once per device, with that device current: the array's device address
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return HOSNWT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return HOSNWT_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return HOSNWT_OK;
}

// quarter-wave table cos(pi m / (2D)), m = 0..D, built on the device; the
// exact values at m = D (0) and m = 2D/3 (1/2) are set as the context's
// host-built table sets them.  Other entries may differ from that table in
// the last bit, so results may differ from hosnwt_transform's in the last
// bits (far inside the transform tolerance).
__global__ void k_noalloc_table(double* q, int D) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > D) return;
  double v = cospi((double)m / (2.0 * (double)D));
  if (m == D) v = 0.0;
  if (D % 3 == 0 && 3 * m == 2 * D) v = 0.5;
  q[m] = v;
}

}  // namespace
}  // namespace hos

using namespace hos;

extern "C" int hosnwt_transform_noalloc(int dir, int cs, int n, int nlines, const double* in,
                                        double* out, void* stream) {
  if ((dir != 1 && dir != -1) || (cs != 0 && cs != 1) || !in || !out || nlines < 1)
    return HOSNWT_ERR_ARG;
  if (n < 5 || n > kNoallocMaxN) return HOSNWT_ERR_ARG;  // sizes beyond the fixed array
  double* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != HOSNWT_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the status returned below covers this call's own launches: clear a
  // launch error an earlier call left on this host thread
  (void)cudaGetLastError();
  double* q = base;
  double* part = base + kTableLen;
  unsigned int* cnt = reinterpret_cast<unsigned int*>(base + kTableLen + kPartLen);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return HOSNWT_ERR_CUDA;
  // the counters must start at zero; the table is rebuilt for this length
  if (cudaMemsetAsync(cnt, 0, sizeof(unsigned int) * kCntLen, st) != cudaSuccess) return HOSNWT_ERR_CUDA;
  k_noalloc_table<<<(n + 255) / 256, 256, 0, st>>>(q, n - 1);
  if (cudaGetLastError() != cudaSuccess) return HOSNWT_ERR_CUDA;
  Tables tb{};
  tb.n1 = n;
  tb.n2 = 1;
  tb.nd1 = n;
  tb.nd2 = 1;
  tb.n3_add = n;
  tb.q_n1 = tb.q_nd1 = tb.q_add = tb.q_n2 = tb.q_nd2 = q;
  tb.nsm = sms > 0 ? sms : 1;
  tb.part = part;
  tb.part_cap = kPartLen;
  tb.cnt = cnt;
  tb.cnt_cap = kCntLen;
  tb.q_const = false;  // the table kernel above runs right before the passes
  double* no_tmp[kMaxJobs] = {};
  XfReq rq[kMaxJobs];
  for (int l0 = 0; l0 < nlines; l0 += kMaxJobs) {
    const int cntl = (nlines - l0 < kMaxJobs) ? nlines - l0 : kMaxJobs;
    for (int i = 0; i < cntl; ++i) {
      XfReq& r = rq[i];
      r.grid = GRID_N;
      r.dir = dir;
      r.csx = cs;
      r.csy = 0;
      r.in = in + (long long)(l0 + i) * n;
      r.in_ld = n;
      r.nin1 = n;
      r.nin2 = 1;
      r.out = out + (long long)(l0 + i) * n;
      r.out_ld = n;
      r.nout1 = n;
      r.nout2 = 1;
      r.scale = 1.0;
    }
    launch_transforms(rq, cntl, tb, no_tmp, st);
  }
  return cudaGetLastError() == cudaSuccess ? HOSNWT_OK : HOSNWT_ERR_CUDA;
}
