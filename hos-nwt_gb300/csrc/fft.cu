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
// GB300 runs FP64 (and conversions between FP64 and FP32) at about 2
// operations per clock per SM, FP32 at 128: in FP64 these passes are bound by
// the FP64 pipe, not by HBM.  So by default the complex DFT runs in
// double-float arithmetic (pairs of FP32 numbers, 48-bit significands, see
// the arithmetic section), on one line per complex sequence: the paired
// form above gets its odd outputs from prefix sums, whose error grows like
// sqrt(N) and lands on the high modes that the HOS orders multiply by k^m;
// the folded form of one line (see the kernel) has no such sums, and its
// errors match the FP64 paired form.  The inputs, weights and scales move
// between FP64 and double-float by integer bit manipulation, so that a pass
// issues about one FP64 instruction per output.  HOSNWT_FFT_DF=0 keeps the
// FP64 paired form.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "hosnwt_internal.h"

namespace hos {

namespace {

constexpr int kFT = 256;           // threads per CTA (8 warps); 512 for Bluestein launches
constexpr int kFTBig = 512;
#ifndef HOSNWT_FFT_MIN_BLOCKS
#define HOSNWT_FFT_MIN_BLOCKS 3    // resident CTAs per SM the register budget is cut for
#endif
constexpr int kFWMax = kFTBig / 32;
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
  int pairs;                 // complex sequences per CTA: line pairs, or lines in double-float
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

// ---------------------------------------------------------------- arithmetic
//
// The FFT core runs on one of two element types of 16 bytes:
//   double2  FP64 complex;
//   dfc      double-float complex: each part is an unevaluated sum hi + lo of
//            two FP32 numbers (|lo| <= ulp(hi) / 2, a 48-bit significand).
// GB300 issues FP32 at 64 times its FP64 rate, and a double-float add or
// product takes 7 to 19 FP32 instructions built on the error-free
// transformations TwoSum (Knuth), FastTwoSum (Dekker) and TwoProd (an FMA
// gives the exact error of a product), as in the double-double arithmetic of
// Dekker (1971) and Hida, Li and Bailey (QD, 2001).  The add is the "sloppy"
// form: its error is bounded by about 2 u^2 (|a| + |b|) with u = 2^-24, which
// is what the normwise error of an FFT needs.  Inside a butterfly the
// results are left unnormalised (lo may grow to a few ulp of hi, the final
// FastTwoSum of each operation is skipped) and cnorm renormalises every
// value that goes to shared memory: a quarter fewer instructions, for
// transform errors about 1.2 times those of normalised arithmetic (numpy
// emulation of both).  Every step is an explicit round-to-nearest
// intrinsic, so that no contraction changes it.
struct __align__(16) dfc {
  float rh, ih, rl, il;  // real hi, imag hi, real lo, imag lo
};
struct dff {
  float h, l;
};

template <typename T>
struct Ar;
template <>
struct Ar<double2> {
  using R = double;
  __host__ __device__ static constexpr double k(double c) { return c; }
};
template <>
struct Ar<dfc> {
  using R = dff;
  __host__ __device__ static constexpr dff k(double c) {
    return dff{static_cast<float>(c), static_cast<float>(c - static_cast<double>(static_cast<float>(c)))};
  }
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ dff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dff dadd(dff a, dff b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return dff{s, __fadd_rn(e, __fadd_rn(a.l, b.l))};
}
__device__ __forceinline__ dff dnorm(dff a) { return fast_two_sum(a.h, a.l); }
__device__ __forceinline__ dff dneg(dff a) { return dff{-a.h, -a.l}; }
// c x
__device__ __forceinline__ dff dmul(dff c, dff x) {
  const float p = __fmul_rn(c.h, x.h);
  float e = __fmaf_rn(c.h, x.h, -p);
  e = __fmaf_rn(c.h, x.l, e);
  e = __fmaf_rn(c.l, x.h, e);
  return dff{p, e};
}
// acc + c x
__device__ __forceinline__ dff dfma(dff c, dff x, dff acc) {
  const float p = __fmul_rn(c.h, x.h);
  const float e1 = __fmaf_rn(c.h, x.h, -p);
  float s, e2;
  two_sum(acc.h, p, s, e2);
  float lo = __fadd_rn(e1, __fadd_rn(e2, acc.l));
  lo = __fmaf_rn(c.h, x.l, lo);
  lo = __fmaf_rn(c.l, x.h, lo);
  return dff{s, lo};
}
// x y + u v
__device__ __forceinline__ dff ddot2(dff x, dff y, dff u, dff v) {
  const float p1 = __fmul_rn(x.h, y.h), p2 = __fmul_rn(u.h, v.h);
  const float e1 = __fmaf_rn(x.h, y.h, -p1), e2 = __fmaf_rn(u.h, v.h, -p2);
  float s, e;
  two_sum(p1, p2, s, e);
  float lo = __fadd_rn(e1, e2);
  lo = __fmaf_rn(x.h, y.l, lo);
  lo = __fmaf_rn(x.l, y.h, lo);
  lo = __fmaf_rn(u.h, v.l, lo);
  lo = __fmaf_rn(u.l, v.h, lo);
  return dff{s, __fadd_rn(lo, e)};
}

// FP64 <-> double-float by bit manipulation: GB300 converts between FP64
// and FP32 at its FP64 rate, the integer pipe is 30 times faster.  The
// split truncates x to hi (24 significant bits) and the next 24 bits to lo,
// then renormalises; |x| below 2^-126 becomes zero (far below the rounding
// of any nonzero entry of a line), infinities and NaN pass to hi.
__device__ __forceinline__ dff d2df(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long m = b & 0xfffffffffffffULL;
  if (e == 0x7ff) return dff{__uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u)), 0.f};
  const int ef = e - 1023 + 127;
  if (ef <= 0) return dff{__uint_as_float(sign), 0.f};
  if (ef >= 255) return dff{__uint_as_float(sign | 0x7f800000u), 0.f};
  const float hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29));
  const unsigned ml = (unsigned)(m & 0x1fffffffu);  // the 29 bits below hi
  if (ml == 0u) return dff{hi, 0.f};
  const int lz = __clz(ml);                          // >= 3
  const int el = e - 1023 - 52 + (31 - lz) + 127;    // exponent of the leading bit of ml
  if (el <= 0) return dff{hi, 0.f};
  const float lo = __uint_as_float(sign | ((unsigned)el << 23) | ((ml << (lz + 1)) >> 9));
  return fast_two_sum(hi, lo);
}
// exact FP64 value of an FP32 number (FP32 subnormals to zero)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0u) return __longlong_as_double((long long)sign);
  const unsigned long long ed = (e == 255u) ? 0x7ffULL : (unsigned long long)(e - 127u + 1023u);
  return __longlong_as_double((long long)(sign | (ed << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}
// hi + lo, exact in FP64 for a normalised pair: one FP64 add
__device__ __forceinline__ double df2d(dff a) { return f2d_bits(a.h) + f2d_bits(a.l); }
__device__ __forceinline__ dff dscale(float s, dff a) { return dff{s * a.h, s * a.l}; }  // s a power of two

__device__ __forceinline__ dff dre(dfc a) { return dff{a.rh, a.rl}; }
__device__ __forceinline__ dff dim(dfc a) { return dff{a.ih, a.il}; }
__device__ __forceinline__ dfc mkc(dff r, dff i) { return dfc{r.h, i.h, r.l, i.l}; }

// complex operations on both element types (the double2 forms are the FP64
// expressions of the pass; each dfc form is its double-float counterpart)
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmi(double2 a) { return make_double2(a.y, -a.x); }  // -i a
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 chalf(double2 a) { return make_double2(0.5 * a.x, 0.5 * a.y); }
__device__ __forceinline__ double2 cfma(double c, double2 x, double2 acc) {  // acc + c x
  return make_double2(fma(c, x.x, acc.x), fma(c, x.y, acc.y));
}
__device__ __forceinline__ double2 csc(double c, double2 x) { return make_double2(c * x.x, c * x.y); }
__device__ __forceinline__ double2 cmulconj(double2 a, double2 c) {  // conj(a) c
  return make_double2(fma(a.x, c.x, a.y * c.y), fma(a.x, c.y, -a.y * c.x));
}
// exp(-i pi / 4) o and exp(-3 i pi / 4) o, r = sqrt(1/2)
__device__ __forceinline__ double2 crot1(double r, double2 o) { return make_double2(r * (o.x + o.y), r * (o.y - o.x)); }
__device__ __forceinline__ double2 crot3(double r, double2 o) {
  return make_double2(r * (o.y - o.x), -r * (o.x + o.y));
}
__device__ __forceinline__ double2 cnorm(double2 a) { return a; }
__device__ __forceinline__ double tre(double2 c) { return c.x; }
__device__ __forceinline__ double tnim(double2 c) { return -c.y; }
__device__ __forceinline__ double2 ldt(const double2* p) { return __ldg(p); }
__device__ __forceinline__ void put_part(double2* e, int part, double v) { reinterpret_cast<double*>(e)[part] = v; }
template <typename T>
__device__ __forceinline__ T czero();
template <>
__device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }

__device__ __forceinline__ dfc cmul(dfc a, dfc b) {
  return mkc(ddot2(dre(a), dre(b), dneg(dim(a)), dim(b)), ddot2(dre(a), dim(b), dim(a), dre(b)));
}
__device__ __forceinline__ dfc cadd(dfc a, dfc b) { return mkc(dadd(dre(a), dre(b)), dadd(dim(a), dim(b))); }
__device__ __forceinline__ dfc csub(dfc a, dfc b) {
  return mkc(dadd(dre(a), dneg(dre(b))), dadd(dim(a), dneg(dim(b))));
}
__device__ __forceinline__ dfc cmi(dfc a) { return dfc{a.ih, -a.rh, a.il, -a.rl}; }
__device__ __forceinline__ dfc cnorm(dfc a) { return mkc(dnorm(dre(a)), dnorm(dim(a))); }
__device__ __forceinline__ dfc cconj(dfc a) { return dfc{a.rh, -a.ih, a.rl, -a.il}; }
__device__ __forceinline__ dfc chalf(dfc a) {
  return dfc{0.5f * a.rh, 0.5f * a.ih, 0.5f * a.rl, 0.5f * a.il};
}
__device__ __forceinline__ dfc cfma(dff c, dfc x, dfc acc) { return mkc(dfma(c, dre(x), dre(acc)), dfma(c, dim(x), dim(acc))); }
__device__ __forceinline__ dfc csc(dff c, dfc x) { return mkc(dmul(c, dre(x)), dmul(c, dim(x))); }
__device__ __forceinline__ dfc cmulconj(dfc a, dfc c) { return cmul(cconj(a), c); }
__device__ __forceinline__ dfc crot1(dff r, dfc o) {
  return mkc(dmul(r, dadd(dre(o), dim(o))), dmul(r, dadd(dim(o), dneg(dre(o)))));
}
__device__ __forceinline__ dfc crot3(dff r, dfc o) {
  return mkc(dmul(r, dadd(dim(o), dneg(dre(o)))), dneg(dmul(r, dadd(dre(o), dim(o)))));
}
__device__ __forceinline__ dff tre(dfc c) { return dre(c); }
__device__ __forceinline__ dff tnim(dfc c) { return dneg(dim(c)); }
__device__ __forceinline__ dfc ldt(const dfc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return dfc{v.x, v.y, v.z, v.w};
}
template <>
__device__ __forceinline__ dfc czero<dfc>() { return dfc{0.f, 0.f, 0.f, 0.f}; }

template <typename T>
__device__ __forceinline__ const T* tab(const double2* p) {
  return reinterpret_cast<const T*>(p);
}

// forward DFT of R points in registers, X_k = sum_t v_t exp(-2 pi i t k / R)
template <typename T>
__device__ __forceinline__ void dft2(T* v) {
  const T a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T>
__device__ __forceinline__ void dft3(T* v) {
  constexpr auto s = Ar<T>::k(0.86602540378443864676);  // sin(2 pi / 3)
  constexpr auto ms = Ar<T>::k(-0.86602540378443864676);
  const T t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const T m = csub(v[0], chalf(t));
  v[0] = cadd(v[0], t);
  v[1] = cfma(s, cmi(d), m);   // m - i s d
  v[2] = cfma(ms, cmi(d), m);  // m + i s d
}

template <typename T>
__device__ __forceinline__ void dft4(T* v) {
  const T a = cadd(v[0], v[2]), b = csub(v[0], v[2]), c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, cmi(d));
  v[3] = csub(b, cmi(d));
}

template <typename T>
__device__ __forceinline__ void dft5(T* v) {
  // cos(2 pi / 5), cos(4 pi / 5), sin(2 pi / 5), sin(4 pi / 5)
  constexpr auto c1 = Ar<T>::k(0.30901699437494742410), c2 = Ar<T>::k(-0.80901699437494742410);
  constexpr auto s1 = Ar<T>::k(0.95105651629515357212), s2 = Ar<T>::k(0.58778525229247312917);
  constexpr auto ms1 = Ar<T>::k(-0.95105651629515357212);
  const T t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const T d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  const T x0 = v[0];
  const T a1 = cfma(c2, t2, cfma(c1, t1, x0));
  const T a2 = cfma(c1, t2, cfma(c2, t1, x0));
  const T b1 = cfma(s2, d2, csc(s1, d1));
  const T b2 = cfma(ms1, d2, csc(s2, d1));
  v[0] = cadd(x0, cadd(t1, t2));
  v[1] = cadd(a1, cmi(b1));
  v[4] = csub(a1, cmi(b1));
  v[2] = cadd(a2, cmi(b2));
  v[3] = csub(a2, cmi(b2));
}

template <typename T>
__device__ __forceinline__ void dft7(T* v) {
  // cos / sin (2 pi q / 7), q = 1, 2, 3
  constexpr auto c1 = Ar<T>::k(0.62348980185873353053), c2 = Ar<T>::k(-0.22252093395631440429);
  constexpr auto c3 = Ar<T>::k(-0.90096886790241912624);
  constexpr auto s1 = Ar<T>::k(0.78183148246802980871), s2 = Ar<T>::k(0.97492791218182360702);
  constexpr auto s3 = Ar<T>::k(0.43388373911755812048);
  constexpr auto ms1 = Ar<T>::k(-0.78183148246802980871), ms3 = Ar<T>::k(-0.43388373911755812048);
  const T x0 = v[0];
  const T t1 = cadd(v[1], v[6]), t2 = cadd(v[2], v[5]), t3 = cadd(v[3], v[4]);
  const T d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
  const T a1 = cfma(c3, t3, cfma(c2, t2, cfma(c1, t1, x0)));
  const T a2 = cfma(c1, t3, cfma(c3, t2, cfma(c2, t1, x0)));
  const T a3 = cfma(c2, t3, cfma(c1, t2, cfma(c3, t1, x0)));
  const T b1 = cfma(s3, d3, cfma(s2, d2, csc(s1, d1)));
  const T b2 = cfma(ms1, d3, cfma(ms3, d2, csc(s2, d1)));
  const T b3 = cfma(s2, d3, cfma(ms1, d2, csc(s3, d1)));
  v[0] = cadd(x0, cadd(t1, cadd(t2, t3)));
  v[1] = cadd(a1, cmi(b1));
  v[6] = csub(a1, cmi(b1));
  v[2] = cadd(a2, cmi(b2));
  v[5] = csub(a2, cmi(b2));
  v[3] = cadd(a3, cmi(b3));
  v[4] = csub(a3, cmi(b3));
}

template <typename T>
__device__ __forceinline__ void dft8(T* v) {
  constexpr auto r = Ar<T>::k(0.70710678118654752440);  // sqrt(1/2)
  T e[4] = {v[0], v[2], v[4], v[6]};
  T o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e);
  dft4(o);
  // o_k *= exp(-i pi k / 4)
  o[1] = crot1(r, o[1]);
  o[2] = cmi(o[2]);
  o[3] = crot3(r, o[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

template <int R, typename T>
__device__ __forceinline__ void dft(T* v) {
  if constexpr (R == 2) dft2(v);
  else if constexpr (R == 3) dft3(v);
  else if constexpr (R == 4) dft4(v);
  else if constexpr (R == 5) dft5(v);
  else if constexpr (R == 7) dft7(v);
  else dft8(v);
}

// x / d with the stage's constant (make_fastdiv): the stage loops divide
// their work index on every iteration, and a plain division by a run-time
// divisor takes about twenty instructions.
__device__ __forceinline__ int operator/(int x, FastDivC f) {
  return (int)(((unsigned long long)__umulhi((unsigned)x, f.m) + (unsigned)x) >> f.s);
}

// One Stockham stage of radix R (R in {2, 3, 4, 5, 7, 8}) on P sequences of
// length L, src -> dst; Ns is the product of the radices of earlier stages.
// Butterfly j takes src[j + t L/R], twiddled by exp(-2 pi i t k / (Ns R))
// with k = j mod Ns, and writes dst[(j - k) R + k + t Ns].
template <int R, typename T>
__device__ void st_small(const T* __restrict__ src, T* __restrict__ dst, int L, int Ns, int P,
                         const T* __restrict__ stw, FastDivC fnb, FastDivC fns) {
  const int nb = L / R;
  const int W = P * nb;
  for (int w = threadIdx.x; w < W; w += blockDim.x) {
    const int p = w / fnb, j = w - p * nb;
    const int off = p * L;
    const int k = j - (j / fns) * Ns;
    T v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = src[pz(off + j + t * nb)];
    if (k != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], ldt(stw + (t - 1) * Ns + k));
    }
    dft<R>(v);
    const int base = off + (j - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; ++t) dst[pz(base + t * Ns)] = cnorm(v[t]);
  }
}

// One Stockham stage of an odd radix R given at run time.  First the inputs
// t and R - t of every butterfly are twiddled and folded in place into
// s_t = v_t + v_{R-t} (slot t) and d_t = v_t - v_{R-t} (slot R - t); then
// each work item forms the outputs o and R - o of one butterfly:
//   X_o = A - i B, X_{R-o} = A + i B,
//   A = v_0 + sum_t s_t cos(2 pi t o / R),  B = sum_t d_t sin(2 pi t o / R).
template <typename T>
__device__ void st_generic(T* __restrict__ src, T* __restrict__ dst, int L, int Ns, int R, int P,
                           const T* __restrict__ tw, const T* __restrict__ stw, FastDivC fnb,
                           FastDivC fh1, FastDivC fh, FastDivC fns) {
  const int nb = L / R, h = (R + 1) / 2;
  const int rs = L / R;
  const int W1 = P * nb * (h - 1);
  for (int w = threadIdx.x; w < W1; w += blockDim.x) {
    const int r = w / fnb;
    const int j = w - r * nb;
    const int p = r / fh1;
    const int t = 1 + r - p * (h - 1);
    const int off = p * L;
    T va = src[pz(off + j + t * nb)], vb = src[pz(off + j + (R - t) * nb)];
    const int k = j - (j / fns) * Ns;
    if (k != 0) {
      va = cmul(va, ldt(stw + (t - 1) * Ns + k));
      vb = cmul(vb, ldt(stw + (R - t - 1) * Ns + k));
    }
    src[pz(off + j + t * nb)] = cnorm(cadd(va, vb));
    src[pz(off + j + (R - t) * nb)] = cnorm(csub(va, vb));
  }
  __syncthreads();
  const int W2 = P * nb * h;
  for (int w = threadIdx.x; w < W2; w += blockDim.x) {
    const int r = w / fnb;
    const int j = w - r * nb;
    const int p = r / fh;
    const int o = r - p * h;
    const int off = p * L;
    const int k = j - (j / fns) * Ns;
    const int base = off + (j - k) * R + k;
    const T v0 = src[pz(off + j)];
    if (o == 0) {
      T a = v0;
      for (int t = 1; t < h; ++t) a = cnorm(cadd(a, src[pz(off + j + t * nb)]));
      dst[pz(base)] = a;
      continue;
    }
    T A = v0, B = czero<T>();
    int q = o;
    for (int t = 1; t < h; ++t) {
      const T c = ldt(tw + q * rs);  // (cos, -sin)(2 pi q / R)
      const T st = src[pz(off + j + t * nb)], dt = src[pz(off + j + (R - t) * nb)];
      A = cnorm(cfma(tre(c), st, A));
      B = cnorm(cfma(tnim(c), dt, B));
      q += o;
      if (q >= R) q -= R;
    }
    dst[pz(base + o * Ns)] = cnorm(cadd(A, cmi(B)));
    dst[pz(base + (R - o) * Ns)] = cnorm(csub(A, cmi(B)));
  }
}

// One in-place stage of radix R on P sequences of length L (stride `ld`
// between sequences): butterfly (b, j) holds elements b S + j + t m, t < R.
// Decimation in frequency: DFT, then twiddle the outputs; in time: twiddle
// the inputs, then DFT.  Each butterfly reads and writes only its own
// elements, so a stage needs no barrier inside it.
template <int R, bool DIF, typename T>
__device__ void ip_stage(T* __restrict__ x, int L, int ld, int S, int P, const T* __restrict__ tw,
                         FastDivC fnb, FastDivC fm) {
  const int m = S / R;
  const int nb = L / R;
  for (int w = threadIdx.x; w < P * nb; w += blockDim.x) {
    const int p = w / fnb, bj = w - p * nb;
    const int blk = bj / fm, j = bj - blk * m;
    const int base = p * ld + blk * S + j;
    T v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = x[pz(base + t * m)];
    if (!DIF && j != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], ldt(tw + (t - 1) * m + j));
    }
    dft<R>(v);
    if (DIF && j != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = cmul(v[t], ldt(tw + (t - 1) * m + j));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) x[pz(base + t * m)] = cnorm(v[t]);
  }
}

// Stages i0 .. i1-1 of the in-place FFT, in the order of its form (DIF:
// stage i, DIT: stage nst-1-i); all of them by default.
template <bool DIF, typename T>
__device__ void ip_fft(const FftInplace& F, T* x, int ld, int P, int i0 = 0, int i1 = -1) {
  const int n = i1 < 0 ? F.nst : i1;
  for (int i = i0; i < n; ++i) {
    const int s = DIF ? i : F.nst - 1 - i;
    int S = F.L;
    for (int q = 0; q < s; ++q) S /= F.rad[q];
    const T* tw = tab<T>(F.tw) + F.off[s];
    const FastDivC& a = F.dnb[s];
    const FastDivC& b = F.dm[s];
    switch (F.rad[s]) {
      case 2: ip_stage<2, DIF>(x, F.L, ld, S, P, tw, a, b); break;
      case 3: ip_stage<3, DIF>(x, F.L, ld, S, P, tw, a, b); break;
      case 4: ip_stage<4, DIF>(x, F.L, ld, S, P, tw, a, b); break;
      case 5: ip_stage<5, DIF>(x, F.L, ld, S, P, tw, a, b); break;
      case 7: ip_stage<7, DIF>(x, F.L, ld, S, P, tw, a, b); break;
      default: ip_stage<8, DIF>(x, F.L, ld, S, P, tw, a, b); break;
    }
    __syncthreads();
  }
}

// Bluestein's first DIF stage when its radix is 8: a sequence's inputs
// j >= D are zero and D < M / 2, so butterfly j (elements j + t m, t < 8,
// m = M / 8) has t >= 4 zero and t = 3 zero for j + 3 m >= D; the
// radix-8 DFT of (a0, a1, a2, a3, 0, 0, 0, 0) takes half the adds of the
// first level.  The padding is never read, so it needs no zero fill.
template <typename T>
__device__ void ip_first_dif8(T* __restrict__ x, int ld, int P, const T* __restrict__ tw, FastDivC fm, int m, int D) {
  constexpr auto r = Ar<T>::k(0.70710678118654752440);
  for (int w = threadIdx.x; w < P * m; w += blockDim.x) {
    const int p = w / fm, j = w - p * m;
    const int base = p * ld + j;
    T a[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) a[t] = (j + t * m < D) ? x[pz(base + t * m)] : czero<T>();
    // dft4 of (x0, x1, 0, 0): x0 + x1, x0 - i x1, x0 - x1, x0 + i x1
    T e[4] = {cadd(a[0], a[2]), cadd(a[0], cmi(a[2])), csub(a[0], a[2]), csub(a[0], cmi(a[2]))};
    T o[4] = {cadd(a[1], a[3]), cadd(a[1], cmi(a[3])), csub(a[1], a[3]), csub(a[1], cmi(a[3]))};
    o[1] = crot1(r, o[1]);
    o[2] = cmi(o[2]);
    o[3] = crot3(r, o[3]);
    T v[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
    if (j != 0) {
#pragma unroll
      for (int t = 1; t < 8; ++t) v[t] = cmul(v[t], ldt(tw + (t - 1) * m + j));
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) x[pz(base + t * m)] = cnorm(v[t]);
  }
}

// Bluestein's last DIT stage when its radix is 8, for outputs k <= kneed <
// 2 m only: butterfly j yields k = j and k = j + m, the first two outputs
// of its radix-8 DFT, and no butterfly with j > kneed is needed.
template <typename T>
__device__ void ip_last_dit8(T* __restrict__ x, int ld, int P, const T* __restrict__ tw, FastDivC fm, int m,
                             int kneed) {
  constexpr auto r = Ar<T>::k(0.70710678118654752440);
  for (int w = threadIdx.x; w < P * m; w += blockDim.x) {
    const int p = w / fm, j = w - p * m;
    if (j > kneed) continue;
    const int base = p * ld + j;
    T v[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) v[t] = x[pz(base + t * m)];
    if (j != 0) {
#pragma unroll
      for (int t = 1; t < 8; ++t) v[t] = cmul(v[t], ldt(tw + (t - 1) * m + j));
    }
    // outputs 0 and 1 of the radix-8 DFT, as dft8 forms them
    const T e0 = cadd(cadd(v[0], v[4]), cadd(v[2], v[6]));
    const T e1 = cadd(csub(v[0], v[4]), cmi(csub(v[2], v[6])));
    const T o0 = cadd(cadd(v[1], v[5]), cadd(v[3], v[7]));
    const T o1 = crot1(r, cadd(csub(v[1], v[5]), cmi(csub(v[3], v[7]))));
    x[pz(base)] = cnorm(cadd(e0, o0));
    if (j + m <= kneed) x[pz(base + m)] = cnorm(cadd(e1, o1));
  }
}

// The turn of Bluestein's convolution in one pass: the last DIF stage, the
// product with the conjugated kernel spectrum h (conj(x) h, in the DIF
// output order) and the first DIT stage.  Both stages have span R and no
// twiddles, so each butterfly keeps its R elements in registers throughout.
template <int R, typename T>
__device__ void ip_turn_r(T* __restrict__ x, int L, int ld, int P, const T* __restrict__ h, FastDivC fnb) {
  const int nb = L / R;
  for (int w = threadIdx.x; w < P * nb; w += blockDim.x) {
    const int p = w / fnb, blk = w - p * nb;
    const int base = p * ld + blk * R;
    T v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = x[pz(base + t)];
    dft<R>(v);
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = cnorm(cmulconj(cnorm(v[t]), ldt(h + blk * R + t)));
    dft<R>(v);
#pragma unroll
    for (int t = 0; t < R; ++t) x[pz(base + t)] = cnorm(v[t]);
  }
}

template <typename T>
__device__ void ip_turn(const FftInplace& F, T* x, int ld, int P, const T* h) {
  const FastDivC& a = F.dnb[F.nst - 1];
  switch (F.rad[F.nst - 1]) {
    case 2: ip_turn_r<2>(x, F.L, ld, P, h, a); break;
    case 3: ip_turn_r<3>(x, F.L, ld, P, h, a); break;
    case 4: ip_turn_r<4>(x, F.L, ld, P, h, a); break;
    case 5: ip_turn_r<5>(x, F.L, ld, P, h, a); break;
    case 7: ip_turn_r<7>(x, F.L, ld, P, h, a); break;
    default: ip_turn_r<8>(x, F.L, ld, P, h, a); break;
  }
  __syncthreads();
}

// Complex FFT of P sequences of length F.L held in a (a <-> b ping-pong);
// returns the buffer that holds the result.
template <typename T>
__device__ T* run_fft(const FftStages& F, T* a, T* b, int P) {
  int Ns = 1;
  for (int s = 0; s < F.nst; ++s) {
    const int R = F.rad[s];
    const T* stw = tab<T>(F.stw) + F.twoff[s];
    const FastDivC &dnb = F.dnb[s], &dns = F.dns[s];
    switch (R) {
      case 2: st_small<2>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      case 3: st_small<3>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      case 4: st_small<4>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      case 5: st_small<5>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      case 7: st_small<7>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      case 8: st_small<8>(a, b, F.L, Ns, P, stw, dnb, dns); break;
      default: st_generic(a, b, F.L, Ns, R, P, tab<T>(F.tw), stw, dnb, F.dh1[s], F.dh[s], dns); break;
    }
    __syncthreads();
    Ns *= R;
    T* t = a;
    a = b;
    b = t;
  }
  return a;
}

// One CTA = `pairs` complex sequences of one job (line pairs, or lines in
// double-float).  Shared memory: two complex buffers of pairs x (D + 1)
// padded elements; the outputs of the CTA's lines (D + 1 each) are staged
// in whichever buffer the FFT leaves free.
// DF: the complex DFT runs in double-float (the job's desc then holds the
// double-float tables) on one line per complex sequence, without the prefix
// sums (see the load loop); the input weights, the pre- and post-processing
// and the output scales stay FP64.
template <int NJ, int NT, bool DF>
__global__ void __launch_bounds__(NT, NT == kFT ? HOSNWT_FFT_MIN_BLOCKS : 1)
    k_fft_pass(const __grid_constant__ FftBatchT<NJ> b) {
  using T = typename std::conditional<DF, dfc, double2>::type;
  extern __shared__ __align__(128) double2 fsm[];
  __shared__ double red[kFWMax][kFMaxLines];
  __shared__ T z0s[kFMaxLines / 2], a0s[kFMaxLines / 2];
  __shared__ __align__(8) uint64_t tma_bar;
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const FftJob& J = b.job[jb];
  const FftDesc& F = *J.desc;
  // P complex sequences per CTA: line pairs, or lines in double-float
  const int D = F.D, P = J.pairs, NL = DF ? P : 2 * P;
  const int line0 = ((int)blockIdx.x - b.start[jb]) * NL;
  const bool blue = (F.mode == FFT_BLUESTEIN);
  const int zld = blue ? F.ip.L : D;  // stride between the pairs' sequences
  T* A = reinterpret_cast<T*>(fsm);
  T* B = A + padded((long long)P * (D + 1));
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
      for (int i = tid; i < J.tma_nbox * J.tma_box_bytes / 8; i += blockDim.x) st[i] = __longlong_as_double(-1LL);
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
  if constexpr (DF) {
    // One line per sequence, from the DFT of length 2D of the even (cos) or
    // odd (sin) extension of the line, folded to length D: with
    // s_j = u_j + u_{D-j}, r_j = u_j - u_{D-j} (and s_0 = 2 (u_0 + u_D),
    // r_0 = 2 (u_0 - u_D)), W = DFT_D(w) gives every output directly:
    //   cos  w_j = 2 (s_j + r_j sin(theta_j)) + 2 i r_j cos(theta_j),
    //        4 C(2m) = Re W_m,   4 C(2m+1) = Im W_m
    //   sin  w_j = 2 (r_j + s_j sin(theta_j)) + 2 i s_j cos(theta_j),  w_0 = 0,
    //        4 S(2m) = -Im W_m,  4 S(2m+1) = Re W_m
    // (the even outputs are the DFT of the symmetric part, the odd ones that
    // of the Hermitian sequence r_j exp(-i theta_j), both real).  Unlike the
    // prefix sums of the paired form, no output accumulates the errors of
    // many others, so the error grows like log N, not sqrt N.
    // the inputs, weights and trigonometric factors in double-float: no
    // FP64 instruction on the way in
    auto Ud = [&](int j) -> dff {
      if (!valid || j < jlo || j >= jend) return dff{0.f, 0.f};
      double v;
      if (tma) {
        const int bx = j / J.tma_by;
        v = stage[(size_t)bx * (J.tma_box_bytes / 8) + (size_t)(j - bx * J.tma_by) * NL + l];
      } else {
        v = __ldg(x + (long long)j * J.in_sk);
      }
      dff d = d2df(v);
      if (wr) d = dmul(d2df(__ldg(wr + (long long)j * J.win_sk)), d);
      return d;
    };
    for (int w = tid; w < NL * D; w += blockDim.x) {
      const int j = w / NL;
      dff ua = Ud(j), ub = Ud(D - j);
      const dfc cs = ldt(tab<dfc>(F.trig) + j);  // (cos, 2 sin)(theta_j)
      dfc v;
      if (j == 0) {
        ua = dmul(d2df(J.e0), ua);
        ub = dmul(d2df(J.eD), ub);
        v = is_sin ? czero<dfc>() : mkc(dscale(4.f, dadd(ua, ub)), dscale(4.f, dadd(ua, dneg(ub))));
      } else {
        const dff sj = dadd(ua, ub), rj = dadd(ua, dneg(ub));
        const dff a = is_sin ? sj : rj, c = is_sin ? rj : sj;
        v = mkc(dfma(dim(cs), a, dscale(2.f, c)), dscale(2.f, dmul(dre(cs), a)));
      }
      if (blue) v = cmul(cnorm(v), ldt(tab<dfc>(F.chirp) + j));  // Bluestein's premultiply
      A[pz(l * zld + j)] = cnorm(v);
    }
    if (blue && F.ip.rad[0] != 8) {
      // the convolution's zero padding (a radix-8 first stage never reads it)
      const int pad = zld - D;
      for (int w = tid; w < P * pad; w += blockDim.x) {
        const int p = w / pad;
        A[pz(p * zld + D + (w - p * pad))] = czero<dfc>();
      }
    }
  } else {
    for (int w = tid; w < NL * D; w += blockDim.x) {
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
      put_part(A + pz((l >> 1) * zld + j), l & 1, t);
    }
  }
  if (!DF && !is_sin) {
    // lanes with the same line: lane = l (mod NL)
    for (int off = 16; off >= NL; off >>= 1) c1 += __shfl_xor_sync(0xffffffffu, c1, off);
    if (lane < NL) red[warp][lane] = c1;
  }
  __syncthreads();

  // ---- the complex DFT of length D of every pair
  T* Z;
  double* O;  // NL x (D + 1) outputs, in the buffer the DFT leaves free
  if (F.mode == FFT_STOCKHAM) {
    Z = run_fft(F.fft, A, B, P);
    O = reinterpret_cast<double*>(Z == A ? B : A);
  } else if (blue && DF) {
    // as below, with the premultiply done by the load loop, the turn in one
    // pass (ip_turn) and the postmultiply by the unpack
    const int M = zld;
    const FftInplace& I = F.ip;
    if (I.rad[0] == 8) {
      ip_first_dif8(A, M, P, tab<T>(I.tw) + I.off[0], I.dm[0], M / 8, D);
      __syncthreads();
      ip_fft<true>(I, A, M, P, 1, I.nst - 1);
    } else {
      ip_fft<true>(I, A, M, P, 0, I.nst - 1);
    }
    ip_turn(I, A, M, P, tab<T>(F.hrev));
    if (I.rad[0] == 8) {
      // the unpack reads outputs k <= D / 2 < M / 4
      ip_fft<false>(I, A, M, P, 1, I.nst - 1);
      ip_last_dit8(A, M, P, tab<T>(I.tw) + I.off[0], I.dm[0], M / 8, D / 2);
      __syncthreads();
    } else {
      ip_fft<false>(I, A, M, P, 1, I.nst);
    }
    Z = A;
    O = nullptr;  // rows in each sequence's free tail, see orow
  } else if (blue) {
    // X_k = conj-chirp_k sum_j (z_j conj-chirp_j) chirp_{k-j}: a cyclic
    // convolution of length M >= 2 D + 2, in place in A
    const int M = zld;
    for (int w = tid; w < P * M; w += blockDim.x) {
      const int j = w % M;
      const int idx = pz(w);
      A[idx] = (j < D) ? cnorm(cmul(A[idx], ldt(tab<T>(F.chirp) + j))) : czero<T>();
    }
    __syncthreads();
    ip_fft<true>(F.ip, A, M, P);
    for (int w = tid; w < P * M; w += blockDim.x) A[pz(w)] = cnorm(cmulconj(A[pz(w)], ldt(tab<T>(F.hrev) + w % M)));
    __syncthreads();
    ip_fft<false>(F.ip, A, M, P);
    for (int w = tid; w < P * D; w += blockDim.x) {
      const int p = w / D, k = w - p * D;
      const int idx = pz(p * M + k);
      A[idx] = cnorm(cmul(ldt(tab<T>(F.chirp) + k), cconj(A[idx])));
    }
    __syncthreads();
    Z = A;
    O = nullptr;  // rows in each pair's free tail, see orow
  } else {
    const int Ls = D - 1;
    for (int w = tid; w < P * Ls; w += blockDim.x) {
      const int p = w / Ls, m = w - p * Ls;
      B[pz(p * Ls + m)] = A[pz(p * D + __ldg(F.gperm + m))];
    }
    if (tid < P) z0s[tid] = A[pz(tid * D)];
    __syncthreads();
    // z now lives in B (permuted) and z0s: A is free for the ping-pong
    T* S1 = run_fft(F.fft, B, A, P);
    T* S2 = (S1 == B) ? A : B;
    if (tid < P) a0s[tid] = S1[pz(tid * Ls)];
    for (int w = tid; w < P * Ls; w += blockDim.x) S2[pz(w)] = cnorm(cmulconj(S1[pz(w)], ldt(tab<T>(F.bconj) + w % Ls)));
    __syncthreads();
    T* Y = run_fft(F.fft, S2, S1, P);
    Z = (Y == A) ? B : A;
    for (int w = tid; w < P * Ls; w += blockDim.x) {
      const int p = w / Ls, n = w - p * Ls;
      Z[pz(p * D + __ldg(F.gscat + n))] = cnorm(cadd(z0s[p], cconj(Y[pz(w)])));
    }
    if (tid < P) Z[pz(tid * D)] = cnorm(cadd(z0s[tid], a0s[tid]));
    __syncthreads();
    O = reinterpret_cast<double*>(Y);
  }

  // output row of line ll: D + 1 doubles
  auto orow = [&](int ll) -> double* {
    if (!blue) return O + (long long)ll * (D + 1);
    if (DF) return reinterpret_cast<double*>(A + pz(ll * zld + D) + 1);
    return reinterpret_cast<double*>(A + pz((ll >> 1) * zld + D) + 1) + (ll & 1) * (D + 1);
  };

  // ---- unpack the two real spectra of each pair; even outputs and the
  // inputs of the odd-output prefix sums go to the output rows
  const int ne = D / 2, no = (D - 1) / 2;
  if constexpr (DF) {
    // outputs scaled in double-float, one FP64 add each to leave it
    const dff s0 = d2df(J.f0), sm = d2df(J.fm), sl = d2df(J.fl);
    for (int w = tid; w < P * (ne + 1); w += blockDim.x) {
      const int p = w / (ne + 1), m = w - p * (ne + 1);
      dfc W = Z[pz(p * zld + m)];
      if (blue) W = cmul(ldt(tab<dfc>(F.chirp) + m), cconj(W));  // Bluestein's postmultiply
      double* o = orow(p);
      const int k = 2 * m;
      o[k] = df2d(dmul(k == 0 ? s0 : (k == D ? sl : sm), is_sin ? dneg(dim(W)) : dre(W)));
      if (m <= no) o[k + 1] = df2d(dmul(k + 1 == D ? sl : sm, is_sin ? dre(W) : dim(W)));
    }
    __syncthreads();
  } else {
    for (int w = tid; w < P * (ne + 1); w += blockDim.x) {
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
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w][tid];
      orow(tid)[1] = 4.0 * s;
    }
    __syncthreads();

    // ---- odd outputs: inclusive prefix sums over O[1], O[3], ..., O[2 no + 1]
    {
      const int n = no + 1;
      const int c = (n + 31) / 32;
      for (int ll = warp; ll < NL; ll += (int)(blockDim.x >> 5)) {
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
  }

  // ---- scale and store (line fastest, like the loads)
  if (valid) {
    double* __restrict__ out = J.out + (long long)line * J.out_sl;
    const double* o = orow(l);
    for (int w = tid; w < NL * J.nout; w += blockDim.x) {
      const int k = w / NL;
      const bool active = (k >= J.klo) && (k < J.khi);
      const double sc = (k == 0) ? J.f0 : ((k == D) ? J.fl : J.fm);
      const double y = active ? (DF ? o[k] : o[k] * sc) : 0.0;  // double-float rows are scaled
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

// HOSNWT_FFT_BIG=0 keeps Bluestein launches at 256 threads per CTA
bool fft_big_ctas() {
  static const bool on = [] {
    const char* e = std::getenv("HOSNWT_FFT_BIG");
    return !(e && e[0] == '0');
  }();
  return on;
}

// HOSNWT_FFT_DF=0 in the environment keeps the complex DFT of the passes in
// FP64 instead of double-float
bool fft_df_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("HOSNWT_FFT_DF");
    return !(e && e[0] == '0');
  }();
  return on;
}

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

// double-float copy of an FP64 table: hi = fl32(x), lo = fl32(x - hi), the
// layout of dfc (real hi, imag hi, real lo, imag lo)
const double2* upload_df(const std::vector<double2>& v, std::vector<void*>& allocs) {
  std::vector<float4> f(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    const float rh = (float)v[i].x, ih = (float)v[i].y;
    f[i] = make_float4(rh, ih, (float)(v[i].x - (double)rh), (float)(v[i].y - (double)ih));
  }
  return reinterpret_cast<const double2*>(upload_vec(f, allocs));
}

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

// FP32 instructions per complex point of a double-float stage of radix R
// (butterfly and twiddle products, lazy renormalisation), from the counts
// of the arithmetic above
double df_stage_cost(int R) {
  switch (R) {
    case 2: return 38.0;
    case 3: return 59.0;
    case 4: return 62.0;
    case 5: return 96.0;
    case 7: return 123.0;
    default: return 88.0;
  }
}

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

// device copy of a table, FP64 or double-float
const double2* upload_tab(const std::vector<double2>& v, bool df, std::vector<void*>& allocs) {
  return df ? upload_df(v, allocs) : upload_vec(v, allocs);
}

// Stockham stages of length L with their twiddles (FP64 or double-float)
bool upload_stages(const std::vector<int>& rad, int L, bool df, std::vector<void*>& allocs, FftStages* f) {
  f->L = L;
  f->nst = (int)rad.size();
  long long ns = 1;
  for (int s = 0; s < f->nst; ++s) {
    const int R = rad[s], h = (R + 1) / 2;
    f->rad[s] = R;
    f->dnb[s] = make_fastdiv((unsigned)(L / R));
    f->dns[s] = make_fastdiv((unsigned)ns);
    f->dh1[s] = make_fastdiv((unsigned)std::max(h - 1, 1));
    f->dh[s] = make_fastdiv((unsigned)h);
    ns *= R;
  }
  f->tw = upload_tab(twiddles(L), df, allocs);
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
  f->stw = upload_tab(stw, df, allocs);
  return f->tw && f->stw;
}

// In-place stages of length L with their twiddles
bool upload_inplace(const std::vector<int>& rad, int L, bool df, std::vector<void*>& allocs, FftInplace* f) {
  f->L = L;
  f->nst = (int)rad.size();
  std::vector<double2> tw;
  int S = L;
  for (int s = 0; s < f->nst; ++s) {
    const int R = rad[s], m = S / R;
    f->rad[s] = R;
    f->off[s] = (int)tw.size();
    f->dnb[s] = make_fastdiv((unsigned)(L / R));
    f->dm[s] = make_fastdiv((unsigned)m);
    for (int q = 1; q < R; ++q)
      for (int j = 0; j < m; ++j) {
        const cld w = unit_root((long long)q * j, S);
        tw.push_back(make_double2((double)w.real(), (double)w.imag()));
      }
    S = m;
  }
  f->tw = upload_tab(tw, df, allocs);
  return f->tw != nullptr;
}

// shared memory of the Bluestein mode must hold the padded convolution
constexpr long long kBlueMaxM = 12400;

// time of the double-float DFT over its FP64 time (FP32 issues 64 times
// faster, a double-float operation takes 7 to 19 FP32 instructions; 0.3 is
// the ratio measured on the steep tank's passes)
constexpr double kDfCost = 0.3;

}  // namespace

bool build_fft_plan(int D, std::vector<void*>& allocs, FftPlanInfo* out) {
  if (D < 8 || !out) return false;
  FftDesc h{}, hd{};  // FP64 and double-float tables
  h.D = D;
  // candidate algorithms and their FP64 instructions per complex DFT
  std::vector<int> rad_s, rad_r, rad_b;
  double cost_s = 1e300, cost_r = 1e300, cost_b = 1e300;
  if (factor_stages(D, rad_s)) cost_s = stages_cost(rad_s, D);
  if (is_prime(D) && factor_stages(D - 1, rad_r)) cost_r = 2.0 * stages_cost(rad_r, D - 1) + 8.0 * (D - 1);
  // Bluestein's length: the cheapest 7-smooth M >= 2 D + 2, by the FP64
  // model for the FP64 tables and by the double-float one for theirs
  int M = 0, M_df = 0;
  double cost_df = 1e300;
  for (long long c = 2LL * D + 2; c <= std::min<long long>(3LL * D, kBlueMaxM); ++c) {
    std::vector<int> r;
    if (!factor_smooth((int)c, r)) continue;
    const double cb = 2.0 * inplace_cost(r, (int)c) + 4.0 * c + 8.0 * D;
    if (cb < cost_b) {
      cost_b = cb;
      M = (int)c;
      rad_b = r;
    }
    double cd = 0.0;
    for (int R : r) cd += df_stage_cost(R);
    cd *= 2.0 * (double)c;
    if (cd < cost_df) {
      cost_df = cd;
      M_df = (int)c;
    }
  }
  double fcost;
  int mode;
  if (cost_s <= cost_r && cost_s <= cost_b) {
    mode = FFT_STOCKHAM;
    fcost = cost_s;
  } else if (cost_r <= cost_b) {
    mode = FFT_RADER;
    fcost = cost_r;
  } else if (M > 0) {
    mode = FFT_BLUESTEIN;
    fcost = cost_b;
  } else {
    return false;
  }
  // host tables shared by both arithmetics
  std::vector<int> gp, gs;
  std::vector<double2> bc, chirp;
  if (mode == FFT_RADER) {
    const int p = D, g = primitive_root(p);
    if (g == 0) return false;
    gp.resize(p - 1);
    gs.resize(p - 1);
    const long long ginv = powmod(g, p - 2, p);
    for (int m = 0; m < p - 1; ++m) {
      gp[m] = (int)powmod(g, m, p);
      gs[m] = (int)powmod(ginv, m, p);
    }
    std::vector<cld> bq(p - 1);
    for (int q = 0; q < p - 1; ++q) bq[q] = unit_root(gs[q], p);
    const std::vector<cld> B = fft_ld(bq);
    bc.resize(p - 1);
    for (int k = 0; k < p - 1; ++k) {
      const cld v = std::conj(B[k]) / (long double)(p - 1);
      bc[k] = make_double2((double)v.real(), (double)v.imag());
    }
  } else if (mode == FFT_BLUESTEIN) {
    // chirp exp(-i pi j^2 / D) (exact phase index j^2 mod 2D)
    chirp.resize(D);
    for (int j = 0; j < D; ++j) {
      const cld w = unit_root((long long)j * j % (2LL * D), 2LL * D);
      chirp[j] = make_double2((double)w.real(), (double)w.imag());
    }
  }
  // (cos, 2 sin)(pi j / D), j = 0..D
  std::vector<double2> trig(D + 1);
  for (int j = 0; j <= D; ++j) {
    const cld w = unit_root(j, 2LL * D);  // exp(-i pi j / D)
    trig[j] = make_double2((double)w.real(), (double)(-2.0L * w.imag()));
  }
  const int* gp_dev = mode == FFT_RADER ? upload_vec(gp, allocs) : nullptr;
  const int* gs_dev = mode == FFT_RADER ? upload_vec(gs, allocs) : nullptr;
  if (mode == FFT_RADER && (!gp_dev || !gs_dev)) return false;
  // the device tables of one arithmetic (the stages are the same; measured:
  // radix-4 stages in double-float, a third of the butterfly's code, made
  // the steep tank's step 10 % slower)
  auto tables = [&](bool df, FftDesc& d) -> bool {
    std::vector<int> r;
    d.D = D;
    d.mode = mode;
    if (mode == FFT_STOCKHAM) {
      if (!factor_stages(D, r) || !upload_stages(r, D, df, allocs, &d.fft)) return false;
    } else if (mode == FFT_RADER) {
      if (!factor_stages(D - 1, r) || !upload_stages(r, D - 1, df, allocs, &d.fft)) return false;
      d.gperm = gp_dev;
      d.gscat = gs_dev;
      d.bconj = upload_tab(bc, df, allocs);
      if (!d.bconj) return false;
    } else {
      // the kernel h_n = conj chirp_|n| on |n| < D of the cyclic length Ml,
      // and its spectrum, stored conjugated over Ml in the DIF output order
      const int Ml = df ? M_df : M;
      if (!factor_smooth(Ml, r) || !upload_inplace(r, Ml, df, allocs, &d.ip)) return false;
      std::vector<cld> hk(Ml, cld(0, 0));
      for (int j = 0; j < D; ++j) {
        const cld w(chirp[j].x, -chirp[j].y);
        hk[j] = w;
        if (j > 0) hk[Ml - j] = w;
      }
      const std::vector<cld> H = fft_ld(hk);
      const std::vector<int> pos = dif_positions(Ml, r);
      std::vector<double2> hrev(Ml);
      for (int k = 0; k < Ml; ++k) {
        const cld v = std::conj(H[k]) / (long double)Ml;
        hrev[pos[k]] = make_double2((double)v.real(), (double)v.imag());
      }
      d.chirp = upload_tab(chirp, df, allocs);
      d.hrev = upload_tab(hrev, df, allocs);
      if (!d.chirp || !d.hrev) return false;
    }
    d.trig = upload_tab(trig, df, allocs);
    return d.trig != nullptr;
  };
  if (!tables(false, h) || !tables(true, hd)) return false;
  std::vector<FftDesc> two{h, hd};
  const FftDesc* dev = upload_vec(two, allocs);
  if (!dev) return false;
  out->D = D;
  out->mode = h.mode;
  out->M = (h.mode == FFT_BLUESTEIN) ? M : 0;
  out->M_df = (h.mode == FFT_BLUESTEIN) ? M_df : 0;
  out->dev = dev;
  out->dev_df = dev + 1;
  // two lines share one complex FFT; pre/post processing about 7 per point
  out->cost_line = 0.5 * fcost + 7.0 * (D + 1);
  // in double-float each line takes a whole complex DFT, at kDfCost of its
  // FP64 time; the pre- and post-processing (FP32 and integer work, one FP64
  // add per output) about 3 per point
  out->cost_line_df = kDfCost * fcost + 3.0 * (D + 1);
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
    const double c = fft_df_enabled() ? f.cost_line_df : f.cost_line;
    if (mode == 1 || c < 0.9 * cost_other) return &f;
  }
  return nullptr;
}

namespace {

size_t fft_smem(const FftPlanInfo& f, int P) {
  if (f.mode == FFT_BLUESTEIN)
    return (size_t)padded((long long)P * (fft_df_enabled() ? f.M_df : f.M)) * sizeof(double2);
  return (size_t)2 * padded((long long)P * (f.D + 1)) * sizeof(double2);
}

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
void setup_tma(FftJob& f, CUtensorMap* map, const FftPlanInfo& plan, int N, bool df) {
  f.tma = 0;
  const int P = f.pairs, NL = df ? P : 2 * P;
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

// complex sequences per CTA: enough butterflies per stage for the warps,
// enough CTAs for the SMs, shared memory within budget; lines-contiguous (y)
// passes take at least four lines so that a warp's loads fill 32-byte sectors
int pick_pairs(const AxisJob& J, const FftPlanInfo& f, int nsm, bool df) {
  const bool ymode = (J.in_sk != 1);
  const int lps = df ? 1 : 2;  // lines per complex sequence
  int P = ymode ? 8 : 4;
  const int Pmin = ymode ? 4 / lps : 1;
  while (P > Pmin) {
    const long long ctas = (J.nlines + (long long)lps * P - 1) / ((long long)lps * P);
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

namespace {

// One prepared launch of the FFT pass kernel.
struct FftLaunch {
  FftBatchT<kMaxJobs> b{};
  size_t smem = 0;
  int total = 0;
  bool big = false;
  bool df = false;
};

// Layout of a batch: threads per CTA (0: the default, 512 for Bluestein
// jobs and 256 otherwise) and the complex sequences per CTA of every job,
// scaled by 2^pshift from pick_pairs.
struct FftLayout {
  int nt = 0;
  int pshift = 0;
};

bool prepare_fft(const AxisBatch& in, const FftPlanInfo* const* plan, const Tables& tb, FftLayout lay, FftLaunch& L) {
  FftBatchT<kMaxJobs>& b = L.b;
  b = FftBatchT<kMaxJobs>{};
  b.njobs = in.njobs;
  b.acc = in.acc;
  L.smem = 0;
  L.total = 0;
  L.df = fft_df_enabled();
  const bool df = L.df;
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
    f.desc = df ? plan[i]->dev_df : plan[i]->dev;
    int P = pick_pairs(J, *plan[i], tb.nsm, df);
    P = lay.pshift >= 0 ? P << lay.pshift : P >> -lay.pshift;
    const int pmax = df ? kFMaxLines : kFMaxLines / 2;
    if (P < 1 || P > pmax || fft_smem(*plan[i], P) > kFftSmemMax) return false;
    f.pairs = P;
    L.smem = std::max(L.smem, fft_smem(*plan[i], f.pairs));
    if (fft_tma_enabled()) setup_tma(f, &b.tmap[i], *plan[i], J.N, df);
    const int nl = df ? f.pairs : 2 * f.pairs;  // lines per CTA
    b.start[i] = L.total;
    L.total += (J.nlines + nl - 1) / nl;
  }
  b.start[b.njobs] = L.total;
  if (lay.nt == 0) {
    // Bluestein's convolution buffer leaves room for one CTA per SM: give
    // it 16 warps to hide the arithmetic latency
    L.big = false;
    for (int i = 0; i < in.njobs; ++i) L.big = L.big || (plan[i]->mode == FFT_BLUESTEIN && fft_big_ctas());
  } else {
    L.big = (lay.nt == kFTBig);
  }
  return true;
}

void launch_prepared(const FftLaunch& L, cudaStream_t st) {
  if (L.total <= 0) return;
  static PerDeviceOnce attr;
  attr.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_fft_capacity(nj, [&](auto c) {
        constexpr int NJ = decltype(c)::value;
        for (const void* k : {(const void*)k_fft_pass<NJ, kFT, false>, (const void*)k_fft_pass<NJ, kFTBig, false>,
                              (const void*)k_fft_pass<NJ, kFT, true>, (const void*)k_fft_pass<NJ, kFTBig, true>})
          cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFftSmemMax);
      });
  });
  with_fft_capacity(L.b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    const FftBatchT<NJ> bb = shrink_fft<NJ>(L.b);
    if (L.big && L.df) launch_pdl(k_fft_pass<NJ, kFTBig, true>, dim3(L.total), dim3(kFTBig), L.smem, st, bb);
    else if (L.big) launch_pdl(k_fft_pass<NJ, kFTBig, false>, dim3(L.total), dim3(kFTBig), L.smem, st, bb);
    else if (L.df) launch_pdl(k_fft_pass<NJ, kFT, true>, dim3(L.total), dim3(kFT), L.smem, st, bb);
    else launch_pdl(k_fft_pass<NJ, kFT, false>, dim3(L.total), dim3(kFT), L.smem, st, bb);
  });
}

// ---- the layout tuner
//
// A batch's signature holds what sets the cost of its launch (per job: the
// plan, the lines and their counts, the axis, whether TMA can stage it).
// While a step graph is captured, launch_fft_jobs records the batches whose
// signature has no decision; fft_tune_run then times every layout of each
// on scratch outputs (threads per CTA 256 or 512, sequences per CTA scaled
// by 1/4 to 2) and keeps the fastest, and the caller captures again.  Only
// the double-float passes are tuned: their arithmetic per line does not
// depend on the layout, so a tuned step computes the same bits.

struct FftTuneRecord {
  std::string sig;
  AxisBatch in;
  const FftPlanInfo* plan[kMaxJobs];
  const Tables* tb;
};

std::mutex g_tune_mu;
std::map<std::string, FftLayout> g_tune_done;  // guarded by g_tune_mu
// batches recorded by this thread's capture, tuned on its own stream (the
// records point into that context's device memory)
thread_local std::vector<FftTuneRecord> g_tune_pending;
thread_local bool g_tune_recording = false;

std::string fft_signature(const AxisBatch& in, const FftPlanInfo* const* plan) {
  std::string s;
  char buf[160];
  for (int i = 0; i < in.njobs; ++i) {
    const AxisJob& J = in.job[i];
    std::snprintf(buf, sizeof buf, "%d:%d:%d:%d:%d:%d:%lld:%lld:%d:%d:%d;", plan[i]->D, plan[i]->mode, J.nlines,
                  J.nin, J.nout, J.N, J.in_sk, J.in_sl, J.win != nullptr ? 1 : 0, J.epi,
                  (int)(reinterpret_cast<uintptr_t>(J.in) % 16));
    s += buf;
  }
  return s;
}

}  // namespace

bool fft_tune_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("HOSNWT_FFT_TUNE");
    return !(e && e[0] == '0');
  }();
  return on && fft_df_enabled();
}

void fft_tune_record(bool on) { g_tune_recording = on; }

int fft_tune_run(cudaStream_t st) {
  std::vector<FftTuneRecord> todo;
  todo.swap(g_tune_pending);
  if (todo.empty()) return 0;
  // one scratch buffer takes the outputs of every candidate launch
  long long ext = 1;
  for (const FftTuneRecord& r : todo)
    for (int i = 0; i < r.in.njobs; ++i) {
      const AxisJob& J = r.in.job[i];
      ext = std::max(ext, (J.nlines - 1) * J.out_sl + (J.nout - 1) * J.out_sk + 1);
    }
  double* scratch = nullptr;
  if (cudaMalloc(&scratch, sizeof(double) * ext) != cudaSuccess) {
    cudaGetLastError();  // no room for the scratch outputs: keep the default layouts
    return 0;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int tuned = 0;
  bool ok = true;
  for (const FftTuneRecord& r : todo) {
    AxisBatch t = r.in;
    for (int i = 0; i < t.njobs; ++i) {
      t.job[i].out = scratch;
      t.job[i].epi = 0;
    }
    FftLayout best;
    float best_ms = 3.4e38f;
    for (int nt : {kFT, kFTBig})
      for (int ps : {-2, -1, 0, 1}) {
        FftLaunch L;
        if (!prepare_fft(t, r.plan, *r.tb, FftLayout{nt, ps}, L) || L.total <= 0) continue;
        launch_prepared(L, st);  // warm-up
        cudaEventRecord(e0, st);
        for (int rep = 0; rep < 3; ++rep) launch_prepared(L, st);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
          ok = false;
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
          best_ms = ms;
          best = FftLayout{nt, ps};
        }
      }
    if (!ok) break;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_done[r.sig] = best;
    ++tuned;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(scratch);
  return ok && cudaGetLastError() == cudaSuccess ? tuned : -1;
}

void launch_fft_jobs(const AxisBatch& in, const FftPlanInfo* const* plan, const Tables& tb, cudaStream_t st) {
  FftLayout lay;
  if (fft_tune_enabled()) {
    const std::string sig = fft_signature(in, plan);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_done.find(sig);
    if (it != g_tune_done.end()) {
      lay = it->second;
    } else if (g_tune_recording) {
      bool seen = false;
      for (const FftTuneRecord& r : g_tune_pending) seen = seen || r.sig == sig;
      if (!seen) {
        FftTuneRecord r;
        r.sig = sig;
        r.in = in;
        for (int i = 0; i < in.njobs; ++i) r.plan[i] = plan[i];
        r.tb = &tb;
        g_tune_pending.push_back(r);
      }
    }
  }
  FftLaunch L;
  if (!prepare_fft(in, plan, tb, lay, L) && !prepare_fft(in, plan, tb, FftLayout{}, L)) return;
  for (int i = 0; i < in.njobs; ++i) g_xform_fmas += (double)in.job[i].nlines * plan[i]->cost_line;
  launch_prepared(L, st);
}

}  // namespace hos
