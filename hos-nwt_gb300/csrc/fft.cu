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
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hosnwt_internal.h"

namespace hos {

namespace {

constexpr int kFT = 256;           // threads per CTA (8 warps)
constexpr int kFW = kFT / 32;
constexpr int kFMaxLines = 16;     // lines per CTA (8 line pairs)

struct FftJob {
  const double* in;
  double* out;
  long long in_sk, in_sl, out_sk, out_sl;
  const double* win;
  long long win_sk, win_sl;
  int nlines, nin, nout;
  int jlo, jhi, klo, khi;
  double w0, wm, wl, s0, sm, sl, gscale;
  int sin_kind;
  int epi;
  int pairs;                 // line pairs per CTA
  const FftDesc* desc;
};

template <int NJ>
struct FftBatchT {
  FftJob job[NJ];
  int start[NJ + 1];
  int njobs;
  AccEpi acc;
};

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

// One Stockham stage of radix R (R in {2, 3, 4, 5, 8}) on P sequences of
// length L, src -> dst; Ns is the product of the radices of earlier stages.
// Butterfly j takes src[j + t L/R], twiddled by exp(-2 pi i t k / (Ns R))
// with k = j mod Ns, and writes dst[(j - k) R + k + t Ns].
template <int R>
__device__ void st_small(const double2* __restrict__ src, double2* __restrict__ dst, int L, int Ns, int P,
                         const double2* __restrict__ tw) {
  const int nb = L / R;
  const int ts = L / (Ns * R);
  const int W = P * nb;
  for (int w = threadIdx.x; w < W; w += kFT) {
    const int p = w / nb, j = w - p * nb;
    const double2* s = src + (long long)p * L;
    double2* d = dst + (long long)p * L;
    const int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = s[j + t * nb];
    if (k != 0) {
      const int step = k * ts;  // t k ts < L for t < R
      int q = step;
#pragma unroll
      for (int t = 1; t < R; ++t) {
        v[t] = cmul(v[t], __ldg(tw + q));
        q += step;
      }
    }
    dft<R>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; ++t) d[base + t * Ns] = v[t];
  }
}

// One Stockham stage of an odd radix R given at run time.  First the inputs
// t and R - t of every butterfly are twiddled and folded in place into
// s_t = v_t + v_{R-t} (slot t) and d_t = v_t - v_{R-t} (slot R - t); then
// each work item forms the outputs o and R - o of one butterfly:
//   X_o = A - i B, X_{R-o} = A + i B,
//   A = v_0 + sum_t s_t cos(2 pi t o / R),  B = sum_t d_t sin(2 pi t o / R).
__device__ void st_generic(double2* __restrict__ src, double2* __restrict__ dst, int L, int Ns, int R, int P,
                           const double2* __restrict__ tw) {
  const int nb = L / R, h = (R + 1) / 2;
  const int ts = L / (Ns * R), rs = L / R;
  const int W1 = P * nb * (h - 1);
  for (int w = threadIdx.x; w < W1; w += kFT) {
    const int j = w % nb;
    const int r = w / nb;
    const int t = 1 + r % (h - 1);
    const int p = r / (h - 1);
    double2* s = src + (long long)p * L;
    double2 va = s[j + t * nb], vb = s[j + (R - t) * nb];
    const int k = j % Ns;
    if (k != 0) {
      va = cmul(va, __ldg(tw + t * k * ts));
      vb = cmul(vb, __ldg(tw + (R - t) * k * ts));
    }
    s[j + t * nb] = cadd(va, vb);
    s[j + (R - t) * nb] = csub(va, vb);
  }
  __syncthreads();
  const int W2 = P * nb * h;
  for (int w = threadIdx.x; w < W2; w += kFT) {
    const int j = w % nb;
    const int r = w / nb;
    const int o = r % h;
    const int p = r / h;
    const double2* s = src + (long long)p * L;
    double2* d = dst + (long long)p * L;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    const double2 v0 = s[j];
    if (o == 0) {
      double2 a = v0;
      for (int t = 1; t < h; ++t) a = cadd(a, s[j + t * nb]);
      d[base] = a;
      continue;
    }
    double2 A = v0, B = make_double2(0.0, 0.0);
    int q = o;
    for (int t = 1; t < h; ++t) {
      const double2 c = __ldg(tw + q * rs);  // (cos, -sin)(2 pi q / R)
      const double2 st = s[j + t * nb], dt = s[j + (R - t) * nb];
      A.x = fma(st.x, c.x, A.x);
      A.y = fma(st.y, c.x, A.y);
      B.x = fma(dt.x, -c.y, B.x);
      B.y = fma(dt.y, -c.y, B.y);
      q += o;
      if (q >= R) q -= R;
    }
    d[base + o * Ns] = make_double2(A.x + B.y, A.y - B.x);
    d[base + (R - o) * Ns] = make_double2(A.x - B.y, A.y + B.x);
  }
}

// Complex FFT of P sequences of length F.L held in a (a <-> b ping-pong);
// returns the buffer that holds the result.
__device__ double2* run_fft(const FftStages& F, double2* a, double2* b, int P) {
  int Ns = 1;
  for (int s = 0; s < F.nst; ++s) {
    const int R = F.rad[s];
    switch (R) {
      case 2: st_small<2>(a, b, F.L, Ns, P, F.tw); break;
      case 3: st_small<3>(a, b, F.L, Ns, P, F.tw); break;
      case 4: st_small<4>(a, b, F.L, Ns, P, F.tw); break;
      case 5: st_small<5>(a, b, F.L, Ns, P, F.tw); break;
      case 8: st_small<8>(a, b, F.L, Ns, P, F.tw); break;
      default: st_generic(a, b, F.L, Ns, R, P, F.tw); break;
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
// buffers of pairs x D and the outputs of 2 pairs lines (D + 1 each).
template <int NJ>
__global__ void __launch_bounds__(kFT) k_fft_pass(const FftBatchT<NJ> b) {
  extern __shared__ __align__(16) double2 fsm[];
  __shared__ double red[kFW][kFMaxLines];
  __shared__ double2 z0s[kFMaxLines / 2], a0s[kFMaxLines / 2];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const FftJob& J = b.job[jb];
  const FftDesc& F = *J.desc;
  const int D = F.D, P = J.pairs, NL = 2 * P;
  const int line0 = ((int)blockIdx.x - b.start[jb]) * NL;
  double2* A = fsm;
  double2* B = A + (long long)P * D;
  double* O = reinterpret_cast<double*>(B + (long long)P * D);  // NL x (D + 1)
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
  auto U = [&](int j) -> double {
    if (!valid || j < jlo || j >= jend) return 0.0;
    double v = __ldg(x + (long long)j * J.in_sk);
    if (wr) v *= __ldg(wr + (long long)j * J.win_sk);
    return v * ((j == 0) ? J.w0 : (j == D ? J.wl : J.wm));
  };
  const bool is_sin = J.sin_kind != 0;
  double c1 = 0.0;
  for (int w = tid; w < NL * D; w += kFT) {
    const int j = w / NL;
    const double ua = U(j), ub = U(D - j);
    const double2 cs = __ldg(F.trig + j);
    double t;
    if (!is_sin) {
      if (j == 0) {
        t = ua + ub;
        c1 += ua - ub;
      } else {
        t = fma(-cs.y, ua - ub, 0.5 * (ua + ub));
        c1 = fma(ua, cs.x, c1);
      }
    } else {
      t = (j == 0) ? 0.0 : fma(cs.y, ua + ub, 0.5 * (ua - ub));
    }
    reinterpret_cast<double*>(A + (long long)(l >> 1) * D + j)[l & 1] = t;
  }
  if (!is_sin) {
    // lanes with the same line: lane = l (mod NL)
    for (int off = 16; off >= NL; off >>= 1) c1 += __shfl_xor_sync(0xffffffffu, c1, off);
    if (lane < NL) red[warp][lane] = c1;
  }
  __syncthreads();

  // ---- the complex DFT of length D of every pair
  double2* Z;
  if (!F.rader) {
    Z = run_fft(F.fft, A, B, P);
  } else {
    const int Ls = D - 1;
    double2* C = reinterpret_cast<double2*>(O);  // P x Ls fits in the output area
    for (int w = tid; w < P * Ls; w += kFT) {
      const int p = w / Ls, m = w - p * Ls;
      B[(long long)p * Ls + m] = A[(long long)p * D + __ldg(F.gperm + m)];
    }
    if (tid < P) z0s[tid] = A[(long long)tid * D];
    __syncthreads();
    double2* S1 = run_fft(F.fft, B, C, P);
    double2* S2 = (S1 == B) ? C : B;
    if (tid < P) a0s[tid] = S1[(long long)tid * Ls];
    for (int w = tid; w < P * Ls; w += kFT) {
      const int m = w % Ls;
      const double2 a = S1[w], c = __ldg(F.bconj + m);
      // conj(a) * c
      S2[w] = make_double2(fma(a.x, c.x, a.y * c.y), fma(a.x, c.y, -a.y * c.x));
    }
    __syncthreads();
    double2* S3 = (S2 == B) ? C : B;
    double2* Y = run_fft(F.fft, S2, S3, P);
    for (int w = tid; w < P * Ls; w += kFT) {
      const int p = w / Ls, n = w - p * Ls;
      const double2 y = Y[w], z0 = z0s[p];
      A[(long long)p * D + __ldg(F.gscat + n)] = make_double2(z0.x + y.x, z0.y - y.y);
    }
    if (tid < P) A[(long long)tid * D] = cadd(z0s[tid], a0s[tid]);
    __syncthreads();
    Z = A;
  }

  // ---- unpack the two real spectra of each pair; even outputs and the
  // inputs of the odd-output prefix sums go to O
  const int ne = D / 2, no = (D - 1) / 2;
  for (int w = tid; w < P * (ne + 1); w += kFT) {
    const int p = w / (ne + 1), m = w - p * (ne + 1);
    const double2 z1 = Z[(long long)p * D + m];
    const double2 z2 = Z[(long long)p * D + (m == 0 ? 0 : D - m)];
    // T_a = (z1 + conj z2) / 2, T_b = (z1 - conj z2) / (2 i)
    const double tr[2] = {0.5 * (z1.x + z2.x), 0.5 * (z1.y + z2.y)};
    const double ti[2] = {0.5 * (z1.y - z2.y), 0.5 * (z2.x - z1.x)};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      double* o = O + (long long)(2 * p + h) * (D + 1);
      if (!is_sin) {
        o[2 * m] = tr[h];
        if (m >= 1 && m <= no) o[2 * m + 1] = -ti[h];
      } else {
        o[2 * m] = -ti[h];
        if (m == 0) {
          if (no >= 0 && D >= 1) o[1] = 0.5 * tr[h];
        } else if (m <= no) {
          o[2 * m + 1] = tr[h];
        }
      }
    }
  }
  if (!is_sin && tid < NL) {
    double s = 0.0;
    for (int w = 0; w < kFW; ++w) s += red[w][tid];
    O[(long long)tid * (D + 1) + 1] = s;
  }
  __syncthreads();

  // ---- odd outputs: inclusive prefix sums over O[1], O[3], ..., O[2 no + 1]
  {
    const int n = no + 1;
    const int c = (n + 31) / 32;
    for (int ll = warp; ll < NL; ll += kFW) {
      double* o = O + (long long)ll * (D + 1) + 1;
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
    const double* o = O + (long long)l * (D + 1);
    for (int w = tid; w < NL * J.nout; w += kFT) {
      const int k = w / NL;
      const bool active = (k >= J.klo) && (k < J.khi);
      const double sc = (k == 0) ? J.s0 : ((k == D) ? J.sl : J.sm);
      const double y = active ? o[k] * sc * J.gscale : 0.0;
      out[(long long)k * J.out_sk] = y;
      if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)k * J.out_sk, y);
    }
  }
}

template <int NJ>
FftBatchT<NJ> shrink_fft(const FftBatchT<kMaxJobs>& b) {
  FftBatchT<NJ> s{};
  for (int i = 0; i < b.njobs; ++i) s.job[i] = b.job[i];
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
bool factor_stages(int L, std::vector<int>& rad) {
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
    if (p > kFftMaxRadix) return false;
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

// Reference DFT of a short sequence in long double (Rader's kernel spectrum).
std::vector<std::complex<long double>> dft_ld(const std::vector<std::complex<long double>>& a) {
  const int n = (int)a.size();
  std::vector<std::complex<long double>> r(n);
  for (int k = 0; k < n; ++k) {
    std::complex<long double> s = 0;
    for (int j = 0; j < n; ++j) {
      const long long q = (long long)j * k % n;
      const long double ang = -2.0L * kPiL * (long double)q / (long double)n;
      s += a[j] * std::complex<long double>(cosl(ang), sinl(ang));
    }
    r[k] = s;
  }
  return r;
}

}  // namespace

bool build_fft_plan(int D, std::vector<void*>& allocs, FftPlanInfo* out) {
  if (D < 8 || !out) return false;
  FftDesc h{};
  h.D = D;
  std::vector<int> rad;
  int L = D;
  double fcost = 0.0;
  if (factor_stages(D, rad)) {
    h.rader = 0;
    fcost = stages_cost(rad, D);
  } else if (is_prime(D) && factor_stages(D - 1, rad)) {
    h.rader = 1;
    L = D - 1;
    fcost = 2.0 * stages_cost(rad, L) + 8.0 * L;
  } else {
    return false;
  }
  h.fft.L = L;
  h.fft.nst = (int)rad.size();
  for (int s = 0; s < h.fft.nst; ++s) h.fft.rad[s] = rad[s];
  h.fft.tw = upload_vec(twiddles(L), allocs);
  if (!h.fft.tw) return false;
  // (cos, sin)(pi j / D), j = 0..D
  std::vector<double2> trig(D + 1);
  for (int j = 0; j <= D; ++j) {
    long double c, s;
    if (j == 0) { c = 1; s = 0; }
    else if (j == D) { c = -1; s = 0; }
    else if (2 * j == D) { c = 0; s = 1; }
    else {
      const long double a = kPiL * (long double)j / (long double)D;
      c = cosl(a);
      s = sinl(a);
    }
    trig[j] = make_double2((double)c, (double)s);
  }
  h.trig = upload_vec(trig, allocs);
  if (!h.trig) return false;
  if (h.rader) {
    const int p = D, g = primitive_root(p);
    if (g == 0) return false;
    std::vector<int> gp(p - 1), gs(p - 1);
    const long long ginv = powmod(g, p - 2, p);
    for (int m = 0; m < p - 1; ++m) {
      gp[m] = (int)powmod(g, m, p);
      gs[m] = (int)powmod(ginv, m, p);
    }
    std::vector<std::complex<long double>> bq(p - 1);
    for (int q = 0; q < p - 1; ++q) {
      const long double ang = -2.0L * kPiL * (long double)gs[q] / (long double)p;
      bq[q] = std::complex<long double>(cosl(ang), sinl(ang));
    }
    const std::vector<std::complex<long double>> B = dft_ld(bq);
    std::vector<double2> bc(p - 1);
    for (int k = 0; k < p - 1; ++k) {
      const std::complex<long double> v = std::conj(B[k]) / (long double)(p - 1);
      bc[k] = make_double2((double)v.real(), (double)v.imag());
    }
    h.gperm = upload_vec(gp, allocs);
    h.gscat = upload_vec(gs, allocs);
    h.bconj = upload_vec(bc, allocs);
    if (!h.gperm || !h.gscat || !h.bconj) return false;
  }
  std::vector<FftDesc> one(1, h);
  const FftDesc* dev = upload_vec(one, allocs);
  if (!dev) return false;
  out->D = D;
  out->dev = dev;
  // two lines share one complex FFT; pre/post processing about 12 per point
  out->cost_line = 0.5 * fcost + 12.0 * (D + 1);
  return true;
}

double fft_line_cost(const FftPlanInfo& f) { return f.cost_line; }

const FftPlanInfo* fft_choice(const AxisJob& J, const Tables& tb, double cost_other) {
  const int mode = fft_mode();
  if (mode == 0) return nullptr;
  const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);
  if (!c1s1 || J.nlines < 32) return nullptr;
  for (int i = 0; i < tb.nfft; ++i) {
    const FftPlanInfo& f = tb.fft[i];
    if (f.D != J.D || !f.dev) continue;
    if (mode == 1 || f.cost_line < 0.9 * cost_other) return &f;
  }
  return nullptr;
}

namespace {

size_t fft_smem(int D, int P) {
  return (size_t)P * D * 2 * sizeof(double2) + (size_t)2 * P * (D + 1) * sizeof(double);
}

// line pairs per CTA: enough butterflies per stage for the 8 warps, enough
// CTAs for the SMs, shared memory within budget; lines-contiguous (y)
// passes take at least two pairs so that a warp's loads fill 32-byte sectors
int pick_pairs(const AxisJob& J, int nsm) {
  const bool ymode = (J.in_sk != 1);
  int P = ymode ? 8 : 4;
  const int Pmin = ymode ? 2 : 1;
  while (P > Pmin) {
    const long long ctas = (J.nlines + 2LL * P - 1) / (2LL * P);
    if (fft_smem(J.D, P) > 200 * 1024) {
      P /= 2;
      continue;
    }
    if (ctas < 2LL * nsm && (long long)(P / 2) * J.D >= 1024) {
      P /= 2;
      continue;
    }
    break;
  }
  while (P > 1 && fft_smem(J.D, P) > 200 * 1024) P /= 2;
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
    f.w0 = J.w0;
    f.wm = J.wm;
    f.wl = J.wl;
    f.s0 = J.s0;
    f.sm = J.sm;
    f.sl = J.sl;
    f.gscale = J.gscale;
    f.sin_kind = (J.off != 0) ? 1 : 0;
    f.epi = J.epi;
    f.desc = plan[i]->dev;
    f.pairs = pick_pairs(J, tb.nsm);
    smem = std::max(smem, fft_smem(J.D, f.pairs));
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
                             210 * 1024);
      });
  });
  with_fft_capacity(b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    launch_pdl(k_fft_pass<NJ>, dim3(total), dim3(kFT), smem, st, shrink_fft<NJ>(b));
  });
}

}  // namespace hos
