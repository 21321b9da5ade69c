// FFT-based transform passes of the HOS-NWT hot path on sm_103a.
//
// Replaces, for the axis passes over many lines (every pass of a 3-D tank),
// the FFTW r2r plans of fourier_FFTW.f90:130-167 (REDFT00 for the cos
// transforms, RODFT00 on the interior for the sin transforms; S2F/F2S
// normalisation fourier_FFTW.f90:175-229 applied as the pass's input weights
// and output scales).
//
// A DCT-I of N = D + 1 points and a DST-I of its D - 1 interior points are
// computed from ONE real DFT of length D (the FFTPACK / Numerical Recipes
// reduction, restated below), and two lines share one complex DFT of length
// D (line a in the real part, line b in the imaginary part).  With
// theta_j = pi j / D and u the weighted input line:
//   cos kind  t_0 = u_0 + u_D,  t_j = (u_j + u_{D-j}) / 2 - sin(theta_j) (u_j - u_{D-j})
//             C(2m) = Re T_m,   C(2m+1) = C(1) - sum_{l=1..m} Im T_l,
//             C(1) = sum_j u_j cos(theta_j)
//   sin kind  t_0 = 0,          t_j = sin(theta_j) (u_j + u_{D-j}) + (u_j - u_{D-j}) / 2
//             S(2m) = -Im T_m,  S(2m+1) = Re T_0 / 2 + sum_{l=1..m} Re T_l
// where T = DFT_D(t).  The odd outputs are prefix sums, done per line by a
// warp with a shuffle scan in a fixed order (the results are deterministic).
// The kernel carries t scaled by 2 / w (w the interior input weight) and the
// unpacked spectra unhalved, so that the input weights, the halvings and the
// output scales become one multiply per output.
//
// The complex DFT runs in shared memory as Stockham autosort stages (natural
// order in and out): radix 2, 3, 4, 5, 8 butterflies in registers, and a
// generic odd radix R (any prime factor up to kFftMaxRadix) whose outputs k
// and R - k come from the folded sums v_t +- v_{R-t}.  A prime D goes through
// Rader's algorithm: with a primitive root g, X(g^-n) = x_0 + (a * b)(n) for
// a_m = x(g^m), b_q = exp(-2 pi i g^-q / D), a cyclic convolution of length
// D - 1 done with two FFTs of that length.
//
// GB300 runs FP64 at about 2 operations per clock per SM, so these passes are
// bound by the FP64 pipe, not by HBM: the design minimises FP64 instructions
// per output (an FFT instead of the O(N^1.5) or O(N^2) sums) and keeps every
// SM busy (one CTA per group of line pairs, 8 warps each).
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hosnwt_internal.h"

namespace hos {

namespace {

constexpr int kFT = 256;           // threads per CTA (8 warps)
#ifndef HOSNWT_FFT_MIN_BLOCKS
#define HOSNWT_FFT_MIN_BLOCKS 3    // resident CTAs per SM the register budget is cut for
#endif
constexpr int kFW = kFT / 32;
constexpr int kFMaxLines = 16;     // lines per CTA (8 line pairs)
constexpr size_t kFftSmemMax = 220 * 1024;  // dynamic shared memory of one CTA

struct FftJob {
  const double* in;
  double* out;
  long long in_sk, in_sl, out_sk, out_sl;
  const double* win;
  long long win_sk, win_sl;
  int nlines, nin, nout;
  int jlo, jhi, klo, khi;
  double e0, eD;             // end input weights relative to the interior weight
  double f0, fm, fl;         // output scales at k = 0, interior k, k = D (times w / 4)
  int sin_kind;
  int epi;
  int pairs;                 // line pairs per CTA
  const FftDesc* desc;
  // TMA staging of a y pass (lines contiguous): the CTA's lines x N points
  // arrive as tma_nbox boxes of tma_by points, tma_box_bytes apart in
  // shared memory, through the job's tensor map
  int tma;
  int tma_by, tma_nbox, tma_box_bytes;
};

template <int NJ>
struct FftBatchT {
  CUtensorMap tmap[NJ];      // 64-byte aligned: first member of a 64-byte aligned struct
  FftJob job[NJ];
  int start[NJ + 1];
  int njobs;
  AccEpi acc;
};

constexpr unsigned kTmaSpinLimit = 1u << 22;  // mbarrier polls before a TMA wait gives up

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Wait for phase 0 of the mbarrier; false after kTmaSpinLimit polls.
__device__ __forceinline__ bool tma_wait(uint64_t* bar) {
  const unsigned a = smem_addr(bar);
  for (unsigned it = 0; it < kTmaSpinLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory index of complex element i of an FFT buffer: one 16-byte
// slot of padding per 8 elements, so that the stride-R writes of the first
// Stockham stages fall in different banks within each quarter warp.
__device__ __forceinline__ int pz(int i) { return i + (i >> 3); }
__host__ __device__ constexpr long long padded(long long n) { return n + (n >> 3) + 1; }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmi(double2 a) { return make_double2(a.y, -a.x); }  // -i a

// forward DFT of R points in registers, X_k = sum_t v_t exp(-2 pi i t k / R)
template <int R>
__device__ __forceinline__ void dft(double2* v);

template <>
__device__ __forceinline__ void dft<2>(double2* v) {
  const double2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<3>(double2* v) {
  const double s = 0.86602540378443864676;  // sin(2 pi / 3)
  const double2 t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const double2 m = make_double2(fma(-0.5, t.x, v[0].x), fma(-0.5, t.y, v[0].y));
  v[0] = cadd(v[0], t);
  v[1] = make_double2(fma(s, d.y, m.x), fma(-s, d.x, m.y));   // m - i s d
  v[2] = make_double2(fma(-s, d.y, m.x), fma(s, d.x, m.y));   // m + i s d
}

template <>
__device__ __forceinline__ void dft<4>(double2* v) {
  const double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, cmi(d));
  v[3] = csub(b, cmi(d));
}

template <>
__device__ __forceinline__ void dft<5>(double2* v) {
  const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;  // cos(2 pi / 5), cos(4 pi / 5)
  const double s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;   // sin(2 pi / 5), sin(4 pi / 5)
  const double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const double2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  const double2 x0 = v[0];
  const double2 a1 = make_double2(fma(c2, t2.x, fma(c1, t1.x, x0.x)), fma(c2, t2.y, fma(c1, t1.y, x0.y)));
  const double2 a2 = make_double2(fma(c1, t2.x, fma(c2, t1.x, x0.x)), fma(c1, t2.y, fma(c2, t1.y, x0.y)));
  const double2 b1 = make_double2(fma(s2, d2.x, s1 * d1.x), fma(s2, d2.y, s1 * d1.y));
  const double2 b2 = make_double2(fma(-s1, d2.x, s2 * d1.x), fma(-s1, d2.y, s2 * d1.y));
  v[0] = cadd(x0, cadd(t1, t2));
  v[1] = cadd(a1, cmi(b1));
  v[4] = csub(a1, cmi(b1));
  v[2] = cadd(a2, cmi(b2));
  v[3] = csub(a2, cmi(b2));
}

template <>
__device__ __forceinline__ void dft<7>(double2* v) {
  // cos / sin (2 pi q / 7), q = 1, 2, 3
  const double c1 = 0.62348980185873353053, c2 = -0.22252093395631440429, c3 = -0.90096886790241912624;
  const double s1 = 0.78183148246802980871, s2 = 0.97492791218182360702, s3 = 0.43388373911755812048;
  const double2 x0 = v[0];
  const double2 t1 = cadd(v[1], v[6]), t2 = cadd(v[2], v[5]), t3 = cadd(v[3], v[4]);
  const double2 d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
  double2 a1, a2, a3, b1, b2, b3;
  a1.x = fma(c3, t3.x, fma(c2, t2.x, fma(c1, t1.x, x0.x)));
  a1.y = fma(c3, t3.y, fma(c2, t2.y, fma(c1, t1.y, x0.y)));
  a2.x = fma(c1, t3.x, fma(c3, t2.x, fma(c2, t1.x, x0.x)));
  a2.y = fma(c1, t3.y, fma(c3, t2.y, fma(c2, t1.y, x0.y)));
  a3.x = fma(c2, t3.x, fma(c1, t2.x, fma(c3, t1.x, x0.x)));
  a3.y = fma(c2, t3.y, fma(c1, t2.y, fma(c3, t1.y, x0.y)));
  b1.x = fma(s3, d3.x, fma(s2, d2.x, s1 * d1.x));
  b1.y = fma(s3, d3.y, fma(s2, d2.y, s1 * d1.y));
  b2.x = fma(-s1, d3.x, fma(-s3, d2.x, s2 * d1.x));
  b2.y = fma(-s1, d3.y, fma(-s3, d2.y, s2 * d1.y));
  b3.x = fma(s2, d3.x, fma(-s1, d2.x, s3 * d1.x));
  b3.y = fma(s2, d3.y, fma(-s1, d2.y, s3 * d1.y));
  v[0] = cadd(x0, cadd(t1, cadd(t2, t3)));
  v[1] = cadd(a1, cmi(b1));
  v[6] = csub(a1, cmi(b1));
  v[2] = cadd(a2, cmi(b2));
  v[5] = csub(a2, cmi(b2));
  v[3] = cadd(a3, cmi(b3));
  v[4] = csub(a3, cmi(b3));
}

template <>
__device__ __forceinline__ void dft<8>(double2* v) {
  const double r = 0.70710678118654752440;  // sqrt(1/2)
  double2 e[4] = {v[0], v[2], v[4], v[6]};
  double2 o[4] = {v[1], v[3], v[5], v[7]};
  dft<4>(e);
  dft<4>(o);
  // o_k *= exp(-i pi k / 4)
  o[1] = make_double2(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x));
  o[2] = cmi(o[2]);
  o[3] = make_double2(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// One Stockham stage of radix R (R in {2, 3, 4, 5, 7, 8}) on P sequences of
// length L, src -> dst; Ns is the product of the radices of earlier stages.
// Butterfly j takes src[j + t L/R], twiddled by exp(-2 pi i t k / (Ns R))
// with k = j mod Ns, and writes dst[(j - k) R + k + t Ns].
template <int R>
__device__ void st_small(const double2* __restrict__ src, double2* __restrict__ dst, int L, int Ns, int P,
                         const double2* __restrict__ stw) {
  const int nb = L / R;
  const int W = P * nb;
  for (int w = threadIdx.x; w < W; w += kFT) {
    const int p = w / nb, j = w - p * nb;
    const int off = p * L;
    const int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = src[pz(off + j + t * nb)];
    if (k != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], __ldg(stw + (t - 1) * Ns + k));
    }
    dft<R>(v);
    const int base = off + (j - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; ++t) dst[pz(base + t * Ns)] = v[t];
  }
}

// One Stockham stage of an odd radix R given at run time.  First the inputs
// t and R - t of every butterfly are twiddled and folded in place into
// s_t = v_t + v_{R-t} (slot t) and d_t = v_t - v_{R-t} (slot R - t); then
// each work item forms the outputs o and R - o of one butterfly:
//   X_o = A - i B, X_{R-o} = A + i B,
//   A = v_0 + sum_t s_t cos(2 pi t o / R),  B = sum_t d_t sin(2 pi t o / R).
__device__ void st_generic(double2* __restrict__ src, double2* __restrict__ dst, int L, int Ns, int R, int P,
                           const double2* __restrict__ tw, const double2* __restrict__ stw) {
  const int nb = L / R, h = (R + 1) / 2;
  const int rs = L / R;
  const int W1 = P * nb * (h - 1);
  for (int w = threadIdx.x; w < W1; w += kFT) {
    const int j = w % nb;
    const int r = w / nb;
    const int t = 1 + r % (h - 1);
    const int p = r / (h - 1);
    const int off = p * L;
    double2 va = src[pz(off + j + t * nb)], vb = src[pz(off + j + (R - t) * nb)];
    const int k = j % Ns;
    if (k != 0) {
      va = cmul(va, __ldg(stw + (t - 1) * Ns + k));
      vb = cmul(vb, __ldg(stw + (R - t - 1) * Ns + k));
    }
    src[pz(off + j + t * nb)] = cadd(va, vb);
    src[pz(off + j + (R - t) * nb)] = csub(va, vb);
  }
  __syncthreads();
  const int W2 = P * nb * h;
  for (int w = threadIdx.x; w < W2; w += kFT) {
    const int j = w % nb;
    const int r = w / nb;
    const int o = r % h;
    const int p = r / h;
    const int off = p * L;
    const int k = j % Ns;
    const int base = off + (j - k) * R + k;
    const double2 v0 = src[pz(off + j)];
    if (o == 0) {
      double2 a = v0;
      for (int t = 1; t < h; ++t) a = cadd(a, src[pz(off + j + t * nb)]);
      dst[pz(base)] = a;
      continue;
    }
    double2 A = v0, B = make_double2(0.0, 0.0);
    int q = o;
    for (int t = 1; t < h; ++t) {
      const double2 c = __ldg(tw + q * rs);  // (cos, -sin)(2 pi q / R)
      const double2 st = src[pz(off + j + t * nb)], dt = src[pz(off + j + (R - t) * nb)];
      A.x = fma(st.x, c.x, A.x);
      A.y = fma(st.y, c.x, A.y);
      B.x = fma(dt.x, -c.y, B.x);
      B.y = fma(dt.y, -c.y, B.y);
      q += o;
      if (q >= R) q -= R;
    }
    dst[pz(base + o * Ns)] = make_double2(A.x + B.y, A.y - B.x);
    dst[pz(base + (R - o) * Ns)] = make_double2(A.x - B.y, A.y + B.x);
  }
}

// One in-place stage of radix R on P sequences of length L (stride `ld`
// between sequences): butterfly (b, j) holds elements b S + j + t m, t < R.
// Decimation in frequency: DFT, then twiddle the outputs; in time: twiddle
// the inputs, then DFT.  Each butterfly reads and writes only its own
// elements, so a stage needs no barrier inside it.
template <int R, bool DIF>
__device__ void ip_stage(double2* __restrict__ x, int L, int ld, int S, int P, const double2* __restrict__ tw) {
  const int m = S / R;
  const int nb = L / R;
  for (int w = threadIdx.x; w < P * nb; w += kFT) {
    const int p = w / nb, bj = w - p * nb;
    const int blk = bj / m, j = bj - blk * m;
    const int base = p * ld + blk * S + j;
    double2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = x[pz(base + t * m)];
    if (!DIF && j != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], __ldg(tw + (t - 1) * m + j));
    }
    dft<R>(v);
    if (DIF && j != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], __ldg(tw + (t - 1) * m + j));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) x[pz(base + t * m)] = v[t];
  }
}

template <bool DIF>
__device__ void ip_fft(const FftInplace& F, double2* x, int ld, int P) {
  for (int i = 0; i < F.nst; ++i) {
    const int s = DIF ? i : F.nst - 1 - i;
    int S = F.L;
    for (int q = 0; q < s; ++q) S /= F.rad[q];
    const double2* tw = F.tw + F.off[s];
    switch (F.rad[s]) {
      case 2: ip_stage<2, DIF>(x, F.L, ld, S, P, tw); break;
      case 3: ip_stage<3, DIF>(x, F.L, ld, S, P, tw); break;
      case 4: ip_stage<4, DIF>(x, F.L, ld, S, P, tw); break;
      case 5: ip_stage<5, DIF>(x, F.L, ld, S, P, tw); break;
      case 7: ip_stage<7, DIF>(x, F.L, ld, S, P, tw); break;
      default: ip_stage<8, DIF>(x, F.L, ld, S, P, tw); break;
    }
    __syncthreads();
  }
}

// Complex FFT of P sequences of length F.L held in a (a <-> b ping-pong);
// returns the buffer that holds the result.
__device__ double2* run_fft(const FftStages& F, double2* a, double2* b, int P) {
  int Ns = 1;
  for (int s = 0; s < F.nst; ++s) {
    const int R = F.rad[s];
    const double2* stw = F.stw + F.twoff[s];
    switch (R) {
      case 2: st_small<2>(a, b, F.L, Ns, P, stw); break;
      case 3: st_small<3>(a, b, F.L, Ns, P, stw); break;
      case 4: st_small<4>(a, b, F.L, Ns, P, stw); break;
      case 5: st_small<5>(a, b, F.L, Ns, P, stw); break;
      case 7: st_small<7>(a, b, F.L, Ns, P, stw); break;
      case 8: st_small<8>(a, b, F.L, Ns, P, stw); break;
      default: st_generic(a, b, F.L, Ns, R, P, F.tw, stw); break;
    }
    __syncthreads();
    Ns *= R;
    double2* t = a;
    a = b;
    b = t;
  }
  return a;
}

// One CTA = `pairs` line pairs of one job.  Shared memory: two complex
// buffers of pairs x (D + 1) padded elements; the outputs of the 2 pairs
// lines (D + 1 each) are staged in whichever buffer the FFT leaves free.
template <int NJ>
__global__ void __launch_bounds__(kFT, HOSNWT_FFT_MIN_BLOCKS) k_fft_pass(const __grid_constant__ FftBatchT<NJ> b) {
  extern __shared__ __align__(128) double2 fsm[];
  __shared__ double red[kFW][kFMaxLines];
  __shared__ double2 z0s[kFMaxLines / 2], a0s[kFMaxLines / 2];
  __shared__ __align__(8) uint64_t tma_bar;
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const FftJob& J = b.job[jb];
  const FftDesc& F = *J.desc;
  const int D = F.D, P = J.pairs, NL = 2 * P;
  const int line0 = ((int)blockIdx.x - b.start[jb]) * NL;
  const bool blue = (F.mode == FFT_BLUESTEIN);
  const int zld = blue ? F.ip.L : D;  // stride between the pairs' sequences
  double2* A = fsm;
  double2* B = A + padded((long long)P * (D + 1));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  pdl_wait();

  // ---- load the lines (line fastest: each thread keeps one line) and
  // form t_j of the real DFT; the cos kind also sums C(1)
  const int l = tid % NL;
  const int line = line0 + l;
  const bool valid = line < J.nlines;
  const double* __restrict__ x = J.in + (long long)(valid ? line : 0) * J.in_sl;
  const double* __restrict__ wr = J.win ? J.win + (long long)(valid ? line : 0) * J.win_sl : nullptr;
  const int jlo = J.jlo, jend = min(J.jhi, J.nin);
  // input j over the interior weight (the end weights enter at j = 0)
  // y passes with TMA: the CTA's NL lines x N points land in the second
  // buffer (unused until the first FFT stage), point-major, one box of
  // tma_by points per tma_box_bytes
  const bool tma = J.tma != 0;
  const double* stage = reinterpret_cast<const double*>(
      (reinterpret_cast<uintptr_t>(B) + 127) & ~static_cast<uintptr_t>(127));
  if (tma) {
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&tma_bar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&tma_bar)),
                   "r"((unsigned)(J.tma_nbox * J.tma_by * NL * 8))
                   : "memory");
      for (int bx = 0; bx < J.tma_nbox; ++bx) {
        const char* dst = reinterpret_cast<const char*>(stage) + (size_t)bx * J.tma_box_bytes;
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(smem_addr(dst)),
            "l"(&b.tmap[jb]), "r"(line0), "r"(bx * J.tma_by), "r"(smem_addr(&tma_bar))
            : "memory");
      }
    }
    // every thread waits; the block decides together, so that the barrier
    // below is reached by all of its threads or by none
    if (__syncthreads_and(tma_wait(&tma_bar) ? 1 : 0) == 0) {
      // a copy that never lands: poison the tile, so that the step's error
      // estimate becomes NaN and the host reports HOSNWT_ERR_NAN
      double* st = const_cast<double*>(stage);
      for (int i = tid; i < J.tma_nbox * J.tma_box_bytes / 8; i += kFT) st[i] = __longlong_as_double(-1LL);
      __syncthreads();
    }
  }
  auto U = [&](int j) -> double {
    if (!valid || j < jlo || j >= jend) return 0.0;
    double v;
    if (tma) {
      const int bx = j / J.tma_by;
      v = stage[(size_t)bx * (J.tma_box_bytes / 8) + (size_t)(j - bx * J.tma_by) * NL + l];
    } else {
      v = __ldg(x + (long long)j * J.in_sk);
    }
    if (wr) v *= __ldg(wr + (long long)j * J.win_sk);
    return v;
  };
  const bool is_sin = J.sin_kind != 0;
  double c1 = 0.0;
  for (int w = tid; w < NL * D; w += kFT) {
    const int j = w / NL;
    double ua = U(j), ub = U(D - j);
    const double2 cs = __ldg(F.trig + j);  // (cos, 2 sin)(theta_j)
    double t;
    if (j == 0) {
      ua *= J.e0;
      ub *= J.eD;
      t = is_sin ? 0.0 : 2.0 * (ua + ub);
      c1 += ua - ub;
    } else if (!is_sin) {
      t = fma(-cs.y, ua - ub, ua + ub);
      c1 = fma(ua, cs.x, c1);
    } else {
      t = fma(cs.y, ua + ub, ua - ub);
    }
    reinterpret_cast<double*>(A + pz((l >> 1) * zld + j))[l & 1] = t;
  }
  if (!is_sin) {
    // lanes with the same line: lane = l (mod NL)
    for (int off = 16; off >= NL; off >>= 1) c1 += __shfl_xor_sync(0xffffffffu, c1, off);
    if (lane < NL) red[warp][lane] = c1;
  }
  __syncthreads();

  // ---- the complex DFT of length D of every pair
  double2* Z;
  double* O;  // NL x (D + 1) outputs, in the buffer the DFT leaves free
  if (F.mode == FFT_STOCKHAM) {
    Z = run_fft(F.fft, A, B, P);
    O = reinterpret_cast<double*>(Z == A ? B : A);
  } else if (blue) {
    // X_k = conj-chirp_k sum_j (z_j conj-chirp_j) chirp_{k-j}: a cyclic
    // convolution of length M >= 2 D + 2, in place in A
    const int M = zld;
    for (int w = tid; w < P * M; w += kFT) {
      const int j = w % M;
      const int idx = pz(w);
      A[idx] = (j < D) ? cmul(A[idx], __ldg(F.chirp + j)) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    ip_fft<true>(F.ip, A, M, P);
    for (int w = tid; w < P * M; w += kFT) {
      const double2 a = A[pz(w)], c = __ldg(F.hrev + w % M);
      A[pz(w)] = make_double2(fma(a.x, c.x, a.y * c.y), fma(a.x, c.y, -a.y * c.x));  // conj(a) c
    }
    __syncthreads();
    ip_fft<false>(F.ip, A, M, P);
    for (int w = tid; w < P * D; w += kFT) {
      const int p = w / D, k = w - p * D;
      const int idx = pz(p * M + k);
      const double2 y = A[idx];
      A[idx] = cmul(__ldg(F.chirp + k), make_double2(y.x, -y.y));
    }
    __syncthreads();
    Z = A;
    O = nullptr;  // rows in each pair's free tail, see orow
  } else {
    const int Ls = D - 1;
    for (int w = tid; w < P * Ls; w += kFT) {
      const int p = w / Ls, m = w - p * Ls;
      B[pz(p * Ls + m)] = A[pz(p * D + __ldg(F.gperm + m))];
    }
    if (tid < P) z0s[tid] = A[pz(tid * D)];
    __syncthreads();
    // z now lives in B (permuted) and z0s: A is free for the ping-pong
    double2* S1 = run_fft(F.fft, B, A, P);
    double2* S2 = (S1 == B) ? A : B;
    if (tid < P) a0s[tid] = S1[pz(tid * Ls)];
    for (int w = tid; w < P * Ls; w += kFT) {
      const int m = w % Ls;
      const double2 a = S1[pz(w)], c = __ldg(F.bconj + m);
      // conj(a) * c
      S2[pz(w)] = make_double2(fma(a.x, c.x, a.y * c.y), fma(a.x, c.y, -a.y * c.x));
    }
    __syncthreads();
    double2* Y = run_fft(F.fft, S2, S1, P);
    Z = (Y == A) ? B : A;
    for (int w = tid; w < P * Ls; w += kFT) {
      const int p = w / Ls, n = w - p * Ls;
      const double2 y = Y[pz(w)], z0 = z0s[p];
      Z[pz(p * D + __ldg(F.gscat + n))] = make_double2(z0.x + y.x, z0.y - y.y);
    }
    if (tid < P) Z[pz(tid * D)] = cadd(z0s[tid], a0s[tid]);
    __syncthreads();
    O = reinterpret_cast<double*>(Y);
  }

  // output row of line ll: D + 1 doubles
  auto orow = [&](int ll) -> double* {
    if (!blue) return O + (long long)ll * (D + 1);
    return reinterpret_cast<double*>(A + pz((ll >> 1) * zld + D) + 1) + (ll & 1) * (D + 1);
  };

  // ---- unpack the two real spectra of each pair; even outputs and the
  // inputs of the odd-output prefix sums go to the output rows
  const int ne = D / 2, no = (D - 1) / 2;
  for (int w = tid; w < P * (ne + 1); w += kFT) {
    const int p = w / (ne + 1), m = w - p * (ne + 1);
    const double2 z1 = Z[pz(p * zld + m)];
    const double2 z2 = Z[pz(p * zld + (m == 0 ? 0 : D - m))];
    // 2 T_a = z1 + conj z2, 2 T_b = (z1 - conj z2) / i: real parts tr,
    // imaginary parts with the sign flipped nti
    const double tr[2] = {z1.x + z2.x, z1.y + z2.y};
    const double nti[2] = {z2.y - z1.y, z1.x - z2.x};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      double* o = orow(2 * p + h);
      if (!is_sin) {
        o[2 * m] = tr[h];
        if (m >= 1 && m <= no) o[2 * m + 1] = nti[h];
      } else {
        o[2 * m] = nti[h];
        if (m == 0) {
          o[1] = 0.5 * tr[h];
        } else if (m <= no) {
          o[2 * m + 1] = tr[h];
        }
      }
    }
  }
  if (!is_sin && tid < NL) {
    double s = 0.0;
    for (int w = 0; w < kFW; ++w) s += red[w][tid];
    orow(tid)[1] = 4.0 * s;
  }
  __syncthreads();

  // ---- odd outputs: inclusive prefix sums over O[1], O[3], ..., O[2 no + 1]
  {
    const int n = no + 1;
    const int c = (n + 31) / 32;
    for (int ll = warp; ll < NL; ll += kFW) {
      double* o = orow(ll) + 1;
      const int i0 = min(lane * c, n), i1 = min(i0 + c, n);
      double s = 0.0;
      for (int i = i0; i < i1; ++i) s += o[2 * i];
      double incl = s;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
      }
      double run = __shfl_up_sync(0xffffffffu, incl, 1);
      if (lane == 0) run = 0.0;
      for (int i = i0; i < i1; ++i) {
        run += o[2 * i];
        o[2 * i] = run;
      }
    }
  }
  __syncthreads();

  // ---- scale and store (line fastest, like the loads)
  if (valid) {
    double* __restrict__ out = J.out + (long long)line * J.out_sl;
    const double* o = orow(l);
    for (int w = tid; w < NL * J.nout; w += kFT) {
      const int k = w / NL;
      const bool active = (k >= J.klo) && (k < J.khi);
      const double sc = (k == 0) ? J.f0 : ((k == D) ? J.fl : J.fm);
      const double y = active ? o[k] * sc : 0.0;
      out[(long long)k * J.out_sk] = y;
      if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)k * J.out_sk, y);
    }
  }
}

template <int NJ>
FftBatchT<NJ> shrink_fft(const FftBatchT<kMaxJobs>& b) {
  FftBatchT<NJ> s{};
  for (int i = 0; i < b.njobs; ++i) {
    s.job[i] = b.job[i];
    s.tmap[i] = b.tmap[i];
  }
  for (int i = 0; i <= b.njobs; ++i) s.start[i] = b.start[i];
  s.njobs = b.njobs;
  s.acc = b.acc;
  return s;
}

template <typename Fn>
void with_fft_capacity(int njobs, Fn&& f) {
  if (njobs <= 1) f(std::integral_constant<int, 1>());
  else if (njobs <= 2) f(std::integral_constant<int, 2>());
  else if (njobs <= 4) f(std::integral_constant<int, 4>());
  else if (njobs <= 8) f(std::integral_constant<int, 8>());
  else f(std::integral_constant<int, kMaxJobs>());
}

// ---------------------------------------------------------------- host side

// HOSNWT_FFT_TMA=0 in the environment keeps the y passes on plain loads
bool fft_tma_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("HOSNWT_FFT_TMA");
    return !(e && e[0] == '0');
  }();
  return on;
}

int fft_mode() {
  static const int m = [] {
    const char* e = std::getenv("HOSNWT_FFT");
    if (!e || !e[0]) return 2;  // auto
    return e[0] == '0' ? 0 : (e[0] == '1' ? 1 : 2);
  }();
  return m;
}

// FP64 instructions per complex point of a stage of radix R (the butterfly,
// plus the twiddle products after the first stage)
double stage_cost(int R, bool first) {
  double bf;
  switch (R) {
    case 2: bf = 2.0; break;
    case 3: bf = 4.7; break;
    case 4: bf = 4.0; break;
    case 5: bf = 7.0; break;
    case 7: bf = 9.5; break;
    case 8: bf = 7.0; break;
    default: bf = R + 3.0; break;
  }
  return bf + (first ? 0.0 : 4.0 * (R - 1) / R);
}

double stages_cost(const std::vector<int>& rad, int L) {
  double c = 0.0;
  for (size_t s = 0; s < rad.size(); ++s) c += stage_cost(rad[s], s == 0);
  return c * L;
}

// Radices of a complex FFT of length L: odd prime factors above 5 first
// (the first stage needs no twiddles), then 8s, a 4 or a 2, then 5s and 3s.
bool factor_stages(int L, std::vector<int>& rad, int maxp = kFftMaxRadix) {
  rad.clear();
  if (L < 2) return false;
  int n = L, twos = 0;
  while (n % 2 == 0) {
    n /= 2;
    ++twos;
  }
  std::vector<int> odd;
  for (int p = 3; (long long)p * p <= n; p += 2)
    while (n % p == 0) {
      odd.push_back(p);
      n /= p;
    }
  if (n > 1) odd.push_back(n);
  for (int p : odd)
    if (p > maxp) return false;
  std::sort(odd.begin(), odd.end(), [](int a, int b2) { return a > b2; });
  for (int p : odd)
    if (p > 5) rad.push_back(p);
  while (twos >= 3) {
    rad.push_back(8);
    twos -= 3;
  }
  if (twos == 2) rad.push_back(4);
  if (twos == 1) rad.push_back(2);
  for (int p : odd)
    if (p <= 5) rad.push_back(p);
  return (int)rad.size() <= kFftMaxSt;
}

bool is_prime(int n) {
  if (n < 2) return false;
  for (int p = 2; (long long)p * p <= n; ++p)
    if (n % p == 0) return false;
  return true;
}

long long powmod(long long a, long long e, long long m) {
  long long r = 1 % m;
  a %= m;
  while (e > 0) {
    if (e & 1) r = r * a % m;
    a = a * a % m;
    e >>= 1;
  }
  return r;
}

int primitive_root(int p) {
  std::vector<int> qs;
  int n = p - 1;
  for (int q = 2; (long long)q * q <= n; ++q)
    if (n % q == 0) {
      qs.push_back(q);
      while (n % q == 0) n /= q;
    }
  if (n > 1) qs.push_back(n);
  for (int g = 2; g < p; ++g) {
    bool ok = true;
    for (int q : qs)
      if (powmod(g, (p - 1) / q, p) == 1) {
        ok = false;
        break;
      }
    if (ok) return g;
  }
  return 0;
}

constexpr long double kPiL = 3.141592653589793238462643383279502884L;

// exp(-2 pi i q / L), q = 0..L-1, exact at the quarter turns
std::vector<double2> twiddles(int L) {
  std::vector<double2> t(L);
  for (int q = 0; q < L; ++q) {
    long double c, s;
    if (4LL * q == 0) { c = 1; s = 0; }
    else if (4LL * q == L) { c = 0; s = 1; }
    else if (2LL * q == L) { c = -1; s = 0; }
    else if (4LL * q == 3LL * L) { c = 0; s = -1; }
    else {
      const long double a = 2.0L * kPiL * (long double)q / (long double)L;
      c = cosl(a);
      s = sinl(a);
    }
    t[q] = make_double2((double)c, (double)-s);
  }
  return t;
}

template <typename T>
T* upload_vec(const std::vector<T>& v, std::vector<void*>& allocs) {
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(v.size(), 1)) != cudaSuccess) return nullptr;
  allocs.push_back(p);
  if (!v.empty() && cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return nullptr;
  return static_cast<T*>(p);
}

using cld = std::complex<long double>;

cld unit_root(long long q, long long n) {  // exp(-2 pi i q / n)
  q %= n;
  if (q < 0) q += n;
  if (q == 0) return cld(1, 0);
  if (4 * q == n) return cld(0, -1);
  if (2 * q == n) return cld(-1, 0);
  if (4 * q == 3 * n) return cld(0, 1);
  const long double a = 2.0L * kPiL * (long double)q / (long double)n;
  return cld(cosl(a), -sinl(a));
}

// Host DFT in long double (forward, exp(-2 pi i j k / n)): recursive
// mixed-radix Cooley-Tukey on the smallest prime factor, for the tables
// of Rader's and Bluestein's kernels.
std::vector<cld> fft_ld(const std::vector<cld>& a) {
  const int n = (int)a.size();
  if (n <= 1) return a;
  int r = n;
  for (int q = 2; (long long)q * q <= n; ++q)
    if (n % q == 0) {
      r = q;
      break;
    }
  std::vector<cld> w(n);
  for (int q = 0; q < n; ++q) w[q] = unit_root(q, n);
  std::vector<cld> out(n);
  if (r == n) {
    for (int k = 0; k < n; ++k) {
      cld acc = 0;
      for (int j = 0; j < n; ++j) acc += a[j] * w[(long long)j * k % n];
      out[k] = acc;
    }
    return out;
  }
  const int m = n / r;
  std::vector<std::vector<cld>> sub(r);
  for (int t = 0; t < r; ++t) {
    std::vector<cld> x(m);
    for (int k = 0; k < m; ++k) x[k] = a[(long long)k * r + t];
    sub[t] = fft_ld(x);
  }
  for (int q = 0; q < r; ++q)
    for (int k = 0; k < m; ++k) {
      const int f = k + q * m;
      cld acc = 0;
      for (int t = 0; t < r; ++t) acc += sub[t][k] * w[(long long)t * f % n];
      out[f] = acc;
    }
  return out;
}

// Radices of a 7-smooth length for the in-place FFT: 8s, a 4 or a 2, then
// 7s, 5s and 3s; false if L has a prime factor above 7.
bool factor_smooth(int L, std::vector<int>& rad) { return factor_stages(L, rad, 7); }

double inplace_cost(const std::vector<int>& rad, int L) {
  double c = 0.0;
  for (size_t s = 0; s < rad.size(); ++s) c += stage_cost(rad[s], s + 1 == rad.size());
  return c * L;
}

// digit-reversed position of frequency k after the in-place DIF stages
std::vector<int> dif_positions(int L, const std::vector<int>& rad) {
  std::vector<int> pos(L);
  for (int k = 0; k < L; ++k) {
    int kk = k, p = 0, span = L;
    for (int R : rad) {
      const int q = kk % R;
      kk /= R;
      span /= R;
      p += q * span;
    }
    pos[k] = p;
  }
  return pos;
}

}  // namespace

namespace {

// Stockham stages of length L with their twiddles
bool upload_stages(const std::vector<int>& rad, int L, std::vector<void*>& allocs, FftStages* f) {
  f->L = L;
  f->nst = (int)rad.size();
  for (int s = 0; s < f->nst; ++s) f->rad[s] = rad[s];
  f->tw = upload_vec(twiddles(L), allocs);
  // stage twiddles exp(-2 pi i t k / (Ns R)) at (t - 1) Ns + k
  std::vector<double2> stw;
  long long Ns = 1;
  for (int st = 0; st < f->nst; ++st) {
    const int R = rad[st];
    f->twoff[st] = (int)stw.size();
    const long long den = Ns * R;
    for (int t = 1; t < R; ++t)
      for (long long k = 0; k < Ns; ++k) {
        const cld w = unit_root((long long)t * k, den);
        stw.push_back(make_double2((double)w.real(), (double)w.imag()));
      }
    Ns *= R;
  }
  f->stw = upload_vec(stw, allocs);
  return f->tw && f->stw;
}

// In-place stages of length L with their twiddles
bool upload_inplace(const std::vector<int>& rad, int L, std::vector<void*>& allocs, FftInplace* f) {
  f->L = L;
  f->nst = (int)rad.size();
  std::vector<double2> tw;
  int S = L;
  for (int s = 0; s < f->nst; ++s) {
    const int R = rad[s], m = S / R;
    f->rad[s] = R;
    f->off[s] = (int)tw.size();
    for (int q = 1; q < R; ++q)
      for (int j = 0; j < m; ++j) {
        const cld w = unit_root((long long)q * j, S);
        tw.push_back(make_double2((double)w.real(), (double)w.imag()));
      }
    S = m;
  }
  f->tw = upload_vec(tw, allocs);
  return f->tw != nullptr;
}

// shared memory of the Bluestein mode must hold the padded convolution
constexpr long long kBlueMaxM = 12400;

}  // namespace

bool build_fft_plan(int D, std::vector<void*>& allocs, FftPlanInfo* out) {
  if (D < 8 || !out) return false;
  FftDesc h{};
  h.D = D;
  // candidate algorithms and their FP64 instructions per complex DFT
  std::vector<int> rad_s, rad_r, rad_b;
  double cost_s = 1e300, cost_r = 1e300, cost_b = 1e300;
  if (factor_stages(D, rad_s)) cost_s = stages_cost(rad_s, D);
  if (is_prime(D) && factor_stages(D - 1, rad_r)) cost_r = 2.0 * stages_cost(rad_r, D - 1) + 8.0 * (D - 1);
  int M = 0;
  for (long long c = 2LL * D + 2; c <= std::min<long long>(3LL * D, kBlueMaxM); ++c) {
    std::vector<int> r;
    if (!factor_smooth((int)c, r)) continue;
    const double cb = 2.0 * inplace_cost(r, (int)c) + 4.0 * c + 8.0 * D;
    if (cb < cost_b) {
      cost_b = cb;
      M = (int)c;
      rad_b = r;
    }
  }
  double fcost;
  if (cost_s <= cost_r && cost_s <= cost_b) {
    h.mode = FFT_STOCKHAM;
    fcost = cost_s;
    if (!upload_stages(rad_s, D, allocs, &h.fft)) return false;
  } else if (cost_r <= cost_b) {
    h.mode = FFT_RADER;
    fcost = cost_r;
    if (!upload_stages(rad_r, D - 1, allocs, &h.fft)) return false;
    const int p = D, g = primitive_root(p);
    if (g == 0) return false;
    std::vector<int> gp(p - 1), gs(p - 1);
    const long long ginv = powmod(g, p - 2, p);
    for (int m = 0; m < p - 1; ++m) {
      gp[m] = (int)powmod(g, m, p);
      gs[m] = (int)powmod(ginv, m, p);
    }
    std::vector<cld> bq(p - 1);
    for (int q = 0; q < p - 1; ++q) bq[q] = unit_root(gs[q], p);
    const std::vector<cld> B = fft_ld(bq);
    std::vector<double2> bc(p - 1);
    for (int k = 0; k < p - 1; ++k) {
      const cld v = std::conj(B[k]) / (long double)(p - 1);
      bc[k] = make_double2((double)v.real(), (double)v.imag());
    }
    h.gperm = upload_vec(gp, allocs);
    h.gscat = upload_vec(gs, allocs);
    h.bconj = upload_vec(bc, allocs);
    if (!h.gperm || !h.gscat || !h.bconj) return false;
  } else if (M > 0) {
    h.mode = FFT_BLUESTEIN;
    fcost = cost_b;
    if (!upload_inplace(rad_b, M, allocs, &h.ip)) return false;
    // chirp exp(-i pi j^2 / D) (exact phase index j^2 mod 2D), the kernel
    // h_n = conj chirp_|n| on |n| < D of the cyclic length M, and its
    // conjugated spectrum over M in the DIF output order
    std::vector<double2> chirp(D);
    std::vector<cld> hk(M, cld(0, 0));
    for (int j = 0; j < D; ++j) {
      const cld w = unit_root((long long)j * j % (2LL * D), 2LL * D);
      chirp[j] = make_double2((double)w.real(), (double)w.imag());
      hk[j] = std::conj(w);
      if (j > 0) hk[M - j] = std::conj(w);
    }
    const std::vector<cld> H = fft_ld(hk);
    const std::vector<int> pos = dif_positions(M, rad_b);
    std::vector<double2> hrev(M);
    for (int k = 0; k < M; ++k) {
      const cld v = std::conj(H[k]) / (long double)M;
      hrev[pos[k]] = make_double2((double)v.real(), (double)v.imag());
    }
    h.chirp = upload_vec(chirp, allocs);
    h.hrev = upload_vec(hrev, allocs);
    if (!h.chirp || !h.hrev) return false;
  } else {
    return false;
  }
  // (cos, 2 sin)(pi j / D), j = 0..D
  std::vector<double2> trig(D + 1);
  for (int j = 0; j <= D; ++j) {
    const cld w = unit_root(j, 2LL * D);  // exp(-i pi j / D)
    trig[j] = make_double2((double)w.real(), (double)(-2.0L * w.imag()));
  }
  h.trig = upload_vec(trig, allocs);
  if (!h.trig) return false;
  std::vector<FftDesc> one(1, h);
  const FftDesc* dev = upload_vec(one, allocs);
  if (!dev) return false;
  out->D = D;
  out->mode = h.mode;
  out->M = (h.mode == FFT_BLUESTEIN) ? M : 0;
  out->dev = dev;
  // two lines share one complex FFT; pre/post processing about 7 per point
  out->cost_line = 0.5 * fcost + 7.0 * (D + 1);
  return true;
}

double fft_line_cost(const FftPlanInfo& f) { return f.cost_line; }

const FftPlanInfo* fft_choice(const AxisJob& J, const Tables& tb, double cost_other) {
  const int mode = fft_mode();
  if (mode == 0) return nullptr;
  const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);
  if (!c1s1 || J.nlines < 32 || J.wm == 0.0) return nullptr;
  for (int i = 0; i < tb.nfft; ++i) {
    const FftPlanInfo& f = tb.fft[i];
    if (f.D != J.D || !f.dev) continue;
    if (mode == 1 || f.cost_line < 0.9 * cost_other) return &f;
  }
  return nullptr;
}

namespace {

size_t fft_smem(const FftPlanInfo& f, int P) {
  if (f.mode == FFT_BLUESTEIN) return (size_t)padded((long long)P * f.M) * sizeof(double2);
  return (size_t)2 * padded((long long)P * (f.D + 1)) * sizeof(double2);
}

// line pairs per CTA: enough butterflies per stage for the 8 warps, enough
// CTAs for the SMs, shared memory within budget; lines-contiguous (y)
// passes take at least two pairs so that a warp's loads fill 32-byte sectors
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn fft_encode_fn() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    return (EncodeTiledFn) nullptr;
  }();
  return fn;
}

// TMA staging of a y pass (lines contiguous, points strided by in_sk): a
// 2-D tensor map of nlines x N doubles and boxes of NL lines x by points.
// Every rule a tiled copy has is checked here, else the pass keeps its
// plain loads: a 16-byte aligned base, a 16-byte multiple stride, an inner
// box extent of NL x 8 bytes (NL even, and every CTA's first line even),
// box smem offsets on 128-byte boundaries inside the second FFT buffer.
void setup_tma(FftJob& f, CUtensorMap* map, const FftPlanInfo& plan, int N) {
  f.tma = 0;
  const int P = f.pairs, NL = 2 * P;
  if (f.in_sl != 1 || f.in_sk <= 1 || f.win || plan.mode == FFT_BLUESTEIN || NL % 2) return;
  if (reinterpret_cast<uintptr_t>(f.in) % 16 != 0 || (f.in_sk * 8) % 16 != 0 || f.in_sk * 8 >= (1LL << 40)) return;
  if (f.nlines < 1 || N < 2) return;
  const int nbox = (N + 255) / 256;
  const int by = (N + nbox - 1) / nbox;
  const long long box_bytes = ((long long)by * NL * 8 + 127) / 128 * 128;
  const long long cap = 16LL * padded((long long)P * (plan.D + 1)) - 127;
  if ((long long)nbox * box_bytes > cap) return;
  const EncodeTiledFn enc = fft_encode_fn();
  if (!enc) return;
  const cuuint64_t dims[2] = {(cuuint64_t)f.nlines, (cuuint64_t)N};
  const cuuint64_t strides[1] = {(cuuint64_t)(f.in_sk * 8)};
  const cuuint32_t box[2] = {(cuuint32_t)NL, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  if (enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(f.in), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return;
  f.tma = 1;
  f.tma_by = by;
  f.tma_nbox = nbox;
  f.tma_box_bytes = (int)box_bytes;
}

int pick_pairs(const AxisJob& J, const FftPlanInfo& f, int nsm) {
  const bool ymode = (J.in_sk != 1);
  int P = ymode ? 8 : 4;
  const int Pmin = ymode ? 2 : 1;
  while (P > Pmin) {
    const long long ctas = (J.nlines + 2LL * P - 1) / (2LL * P);
    if (fft_smem(f, P) > kFftSmemMax) {
      P /= 2;
      continue;
    }
    if (ctas < 2LL * nsm && (long long)(P / 2) * J.D >= 1024) {
      P /= 2;
      continue;
    }
    break;
  }
  while (P > 1 && fft_smem(f, P) > kFftSmemMax) P /= 2;
  return P;
}

}  // namespace

void launch_fft_jobs(const AxisBatch& in, const FftPlanInfo* const* plan, const Tables& tb, cudaStream_t st) {
  FftBatchT<kMaxJobs> b{};
  b.njobs = in.njobs;
  b.acc = in.acc;
  size_t smem = 0;
  int total = 0;
  for (int i = 0; i < in.njobs; ++i) {
    const AxisJob& J = in.job[i];
    FftJob& f = b.job[i];
    f.in = J.in;
    f.out = J.out;
    f.in_sk = J.in_sk;
    f.in_sl = J.in_sl;
    f.out_sk = J.out_sk;
    f.out_sl = J.out_sl;
    f.win = J.win;
    f.win_sk = J.win_sk;
    f.win_sl = J.win_sl;
    f.nlines = J.nlines;
    f.nin = J.nin;
    f.nout = J.nout;
    f.jlo = J.jlo;
    f.jhi = J.jhi;
    f.klo = J.klo;
    f.khi = J.khi;
    // the kernel's outputs are 4 / wm times the transform
    f.e0 = J.w0 / J.wm;
    f.eD = J.wl / J.wm;
    f.f0 = 0.25 * J.wm * J.s0 * J.gscale;
    f.fm = 0.25 * J.wm * J.sm * J.gscale;
    f.fl = 0.25 * J.wm * J.sl * J.gscale;
    f.sin_kind = (J.off != 0) ? 1 : 0;
    f.epi = J.epi;
    f.desc = plan[i]->dev;
    f.pairs = pick_pairs(J, *plan[i], tb.nsm);
    smem = std::max(smem, fft_smem(*plan[i], f.pairs));
    if (fft_tma_enabled()) setup_tma(f, &b.tmap[i], *plan[i], J.N);
    b.start[i] = total;
    total += (J.nlines + 2 * f.pairs - 1) / (2 * f.pairs);
    g_xform_fmas += (double)J.nlines * plan[i]->cost_line;
  }
  b.start[b.njobs] = total;
  if (total <= 0) return;
  static PerDeviceOnce attr;
  attr.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_fft_capacity(nj, [&](auto c) {
        cudaFuncSetAttribute(k_fft_pass<decltype(c)::value>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kFftSmemMax);
      });
  });
  with_fft_capacity(b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    launch_pdl(k_fft_pass<NJ>, dim3(total), dim3(kFT), smem, st, shrink_fft<NJ>(b));
  });
}

}  // namespace hos
