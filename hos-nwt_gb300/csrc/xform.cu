// Spectral transforms of the HOS-NWT hot path on sm_103a.
//
// Replaces the FFTW r2r plans of fourier_FFTW.f90:89-653 (DCT_FFTW,
// IDCT_FFTW, DCT_FFTW_big, IDCT_FFTW_big, DCT_FFTW_add, IDCT_FFTW_add).
// The lengths of the dealiased grid, Nd = ((p+1) n)/2 (common_vars.f90:40-41),
// have large prime factors, so each pass is computed as an exact FP64 sum
// over a quarter-wave twiddle table indexed with integer arithmetic.  That
// works for every length and kind and keeps the normalisation fused.
//
// On GB300 the FP64 pipe (about 1.2 TFLOP/s) is the bound of these passes,
// not HBM: an x pass spreads one line over many CTAs (8 warps split the sum,
// lanes own outputs), a y pass gives one row per lane (coalesced loads,
// warp-uniform twiddles) and several outputs per thread.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include "hosnwt_internal.h"

namespace hos {

namespace {

__device__ __forceinline__ double twiddle(const double* __restrict__ q, int D, int m) {
  // m in [0, 4D): cos(pi*m/(2D)) from the quarter-wave table
  int mm = (m > 2 * D) ? 4 * D - m : m;
  return (mm > D) ? -__ldg(q + (2 * D - mm)) : __ldg(q + mm);
}

__device__ __forceinline__ int mod4d(long long v, int D4) {
  long long r = v % D4;
  return (int)(r < 0 ? r + D4 : r);
}

// input j of a first-pass line, times the optional weight
__device__ __forceinline__ double in_at(const double* __restrict__ x, long long sk,
                                       const double* __restrict__ w, long long wsk, int j) {
  const double v = __ldg(x + (long long)j * sk);
  return w ? v * __ldg(w + (long long)j * wsk) : v;
}

constexpr int kXThreads = 256;   // 8 warps
constexpr int kXWarps = kXThreads / 32;
constexpr int kMaxPairChunk = 1024;  // staged terms per CTA

__device__ __forceinline__ double twiddle_s(const double* q, int D, int m) {
  int mm = (m > 2 * D) ? 4 * D - m : m;
  return (mm > D) ? -q[2 * D - mm] : q[mm];
}

// x pass: one CTA = (job, line, tile of 32 lane outputs, chunk of the sum).
// The quarter-wave table of the job and the CTA's chunk of inputs are staged
// in shared memory; lanes own outputs (twiddles are gathered from shared
// memory, inputs are broadcast), the 8 warps split the chunk, and the chunks
// of one tile are combined in a fixed order by the last CTA to arrive.
//   mode 0: direct sum over the interior terms plus the two end terms
//   mode 1: output symmetry: lane k accumulates even-j and odd-j sums E, O
//           and writes out[k] and out[D-k] (full outputs, D = N-1)
//   mode 2: input symmetry: terms are pairs (j, D-j) staged as
//           u = x_j + x_{D-j}, v = x_j - x_{D-j} (outputs k <= D/2)
template <int NJ>
__global__ void __launch_bounds__(kXThreads) axis_pass_lanes_k(const AxisBatchT<NJ> b) {
  extern __shared__ double smem[];
  __shared__ double red[kXWarps][32][2];
  __shared__ bool amlast;
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  int local = blockIdx.x - b.start[jb];
  const int chunk_id = local % J.nchunk;
  local /= J.nchunk;
  const int tile = local % J.ntile;
  const int line = local / J.ntile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = tile * 32 + lane;
  const int D = J.D, D4 = 4 * D;
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const int kk = J.ak * k + J.bk;
  const int inc = mod4d((long long)J.aj * kk, D4);
  const bool lane_on = k < J.nlane;
  const long long sk = J.in_sk;
  const double* __restrict__ wr = J.win ? J.win + (long long)line * J.win_sl : nullptr;

  double* q = smem;                    // D + 1 table entries
  double* su = smem + (D + 1);         // staged inputs (or u)
  double* sv = su + kMaxPairChunk;     // v (mode 2)
  if (b.early)
    for (int t = threadIdx.x; t <= D; t += kXThreads) q[t] = __ldg(J.q + t);
  pdl_wait();
  if (!b.early)
    for (int t = threadIdx.x; t <= D; t += kXThreads) q[t] = __ldg(J.q + t);
  const int ca = J.ta + chunk_id * J.chunk;
  const int cb = min(J.tb, ca + J.chunk);
  // cos: even k pairs with u; sin: even k pairs with v (mode 2)
  const bool use_v = (J.mode == 2) && (((k & 1) == 0) != (J.off == 0));
  double e = 0.0, o = 0.0;  // mode 1: even / odd j sums; else e only
  for (int sa = ca; sa < cb; sa += kMaxPairChunk) {
    const int sb = min(cb, sa + kMaxPairChunk);
    __syncthreads();  // previous stage consumed
    if (J.mode == 2) {
      for (int t = threadIdx.x; t < sb - sa; t += kXThreads) {
        const int j = sa + t;
        const double xa = in_at(x, sk, wr, J.win_sk, j);
        const double xb = in_at(x, sk, wr, J.win_sk, D - j);
        su[t] = xa + xb;
        sv[t] = xa - xb;
      }
    } else {
      for (int t = threadIdx.x; t < sb - sa; t += kXThreads) su[t] = in_at(x, sk, wr, J.win_sk, sa + t);
    }
    __syncthreads();
    const int len = sb - sa;
    const int per = (len + kXWarps - 1) / kXWarps;
    const int ja = sa + warp * per;
    const int jz = min(sb, ja + per);
    if (lane_on && jz > ja) {
      int m = mod4d((long long)(J.aj * ja + J.bj) * kk + J.off, D4);
      if (J.mode == 1) {
        int j = ja;
        if (j & 1) {  // align to an even j
          o = fma(su[j - sa], twiddle_s(q, D, m), o);
          m += inc;
          if (m >= D4) m -= D4;
          ++j;
        }
        for (; j + 1 < jz; j += 2) {
          const double te = twiddle_s(q, D, m);
          m += inc;
          if (m >= D4) m -= D4;
          const double to = twiddle_s(q, D, m);
          m += inc;
          if (m >= D4) m -= D4;
          e = fma(su[j - sa], te, e);
          o = fma(su[j + 1 - sa], to, o);
        }
        if (j < jz) e = fma(su[j - sa], twiddle_s(q, D, m), e);
      } else {
        const double* sp = use_v ? sv : su;
        double e2 = 0.0;
        int j = ja;
        for (; j + 1 < jz; j += 2) {
          const double t0 = twiddle_s(q, D, m);
          m += inc;
          if (m >= D4) m -= D4;
          const double t1 = twiddle_s(q, D, m);
          m += inc;
          if (m >= D4) m -= D4;
          e = fma(sp[j - sa], t0, e);
          e2 = fma(sp[j + 1 - sa], t1, e2);
        }
        if (j < jz) e = fma(sp[j - sa], twiddle_s(q, D, m), e);
        e += e2;
      }
    }
  }
  if (cb <= ca) __syncthreads();  // table staged even when this CTA has no terms
  e *= J.wm;
  o *= J.wm;
  // end terms and the unpaired middle term, once per tile (chunk 0, warp 0)
  if (chunk_id == 0 && warp == 0 && lane_on) {
    const int j_end = min(J.jhi, J.nin);
    if (J.mode == 2) {
      if (J.jlo == 0) {  // pair (0, D) with the end weight
        const double xa = in_at(x, sk, wr, J.win_sk, 0), xb = in_at(x, sk, wr, J.win_sk, D);
        const double t = ((k & 1) == 0) ? xa + xb : xa - xb;
        e = fma(J.w0 * t, twiddle_s(q, D, mod4d((long long)J.bj * kk + J.off, D4)), e);
      }
      if ((D & 1) == 0) {
        const int jm = D / 2;
        if (jm >= J.jlo && jm < J.jhi && jm > 0) {
          const int mm = mod4d((long long)(J.aj * jm + J.bj) * kk + J.off, D4);
          e = fma(J.wm * in_at(x, sk, wr, J.win_sk, jm), twiddle_s(q, D, mm), e);
        }
      }
    } else {
      if (J.jlo == 0 && 0 < j_end) {
        const int mm = mod4d((long long)J.bj * kk + J.off, D4);
        e = fma(J.w0 * in_at(x, sk, wr, J.win_sk, 0), twiddle_s(q, D, mm), e);
      }
      const int jl = J.N - 1;
      if (jl > 0 && jl >= J.jlo && jl < j_end) {
        const int mm = mod4d((long long)(J.aj * jl + J.bj) * kk + J.off, D4);
        const double t = J.wl * in_at(x, sk, wr, J.win_sk, jl) * twiddle_s(q, D, mm);
        if (J.mode == 1 && (jl & 1)) o += t;
        else e += t;
      }
    }
  }
  red[warp][lane][0] = e;
  red[warp][lane][1] = o;
  __syncthreads();
  double E = 0.0, O = 0.0;
  if (warp == 0) {
#pragma unroll
    for (int w = 0; w < kXWarps; ++w) {
      E += red[w][lane][0];
      O += red[w][lane][1];
    }
  }
  if (J.nchunk > 1) {
    double* pp = J.part + ((long long)(line * J.ntile + tile) * J.nchunk) * 64;
    if (warp == 0) {
      pp[chunk_id * 64 + 2 * lane] = E;
      pp[chunk_id * 64 + 2 * lane + 1] = O;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned int* c = J.cnt + (line * J.ntile + tile);
      const unsigned int t = atomicAdd(c, 1u);
      amlast = (t == (unsigned int)J.nchunk - 1);
      if (amlast) *c = 0u;
    }
    __syncthreads();
    if (!amlast) return;
    if (warp == 0) {
      E = 0.0;
      O = 0.0;
      for (int c = 0; c < J.nchunk; ++c) {
        E += __ldcg(pp + c * 64 + 2 * lane);
        O += __ldcg(pp + c * 64 + 2 * lane + 1);
      }
    }
  }
  if (warp != 0 || !lane_on) return;
  const double g = J.gscale;
  auto scale = [&](int kq) { return (kq == 0) ? J.s0 : ((kq == J.N - 1) ? J.sl : J.sm); };
  auto active = [&](int kq) { return kq >= J.klo && kq < J.khi; };
  double* out = J.out + (long long)line * J.out_sl;
  if (J.mode == 1) {
    const bool is_sin = (J.off != 0);
    const double yk = E + O;
    const double yr = is_sin ? (O - E) : (E - O);
    if (k < J.nout) {
      const double v = active(k) ? yk * scale(k) * g : 0.0;
      out[(long long)k * J.out_sk] = v;
      if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)k * J.out_sk, v);
    }
    const int kr = D - k;
    if (kr != k && kr < J.nout) {
      const double v = active(kr) ? yr * scale(kr) * g : 0.0;
      out[(long long)kr * J.out_sk] = v;
      if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)kr * J.out_sk, v);
    }
  } else {
    if (k < J.nout) {
      const double v = active(k) ? E * scale(k) * g : 0.0;
      out[(long long)k * J.out_sk] = v;
      if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)k * J.out_sk, v);
    }
  }
}

constexpr int kYThreads = 64;
constexpr int kYR = 8;  // outputs per thread

// y pass: one thread = one line (consecutive lines are contiguous in memory)
// and kYR lane outputs; twiddles are warp-uniform.  The two symmetries of
// the x pass halve the FP64 work of REDFT00 / RODFT00 kinds:
//   mode 1: lane output k (k <= D/2) keeps even-j and odd-j sums E, O and
//           writes out[k] and out[D-k]
//   mode 2: inputs are paired, u = x_j + x_{D-j}, v = x_j - x_{D-j}
//           (outputs k <= D/2)
// kYR consecutive twiddles of a y row (rows are 64-byte aligned)
__device__ __forceinline__ void row8(const double* __restrict__ p, double (&t)[kYR]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < kYR / 2; ++i) {
    const double2 v = __ldg(q + i);
    t[2 * i] = v.x;
    t[2 * i + 1] = v.y;
  }
}

template <int NJ>
__global__ void __launch_bounds__(kYThreads) axis_pass_lanes_line(const AxisBatchT<NJ> b) {
  pdl_wait();
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int local = blockIdx.x - b.start[jb];
  const int nlb = (J.nlines + kYThreads - 1) / kYThreads;
  const int kgrp = local / nlb;
  const int lb = local - kgrp * nlb;
  const int line = lb * kYThreads + threadIdx.x;
  if (line >= J.nlines) return;
  const int k0 = kgrp * kYR;
  const int D = J.D, D4 = 4 * D;
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const long long sk = J.in_sk;
  // input weights (a y pass that runs first reads them along y)
  const double* __restrict__ wr = J.win ? J.win + (long long)line * J.win_sl : nullptr;
  auto X = [&](int j) { return in_at(x, sk, wr, J.win_sk, j); };
  const int j_end = min(J.jhi, J.nin);
  const bool is_sin = (J.off != 0);
  double* out = J.out + (long long)line * J.out_sl;
  auto put = [&](int k, double v) {
    if (k >= J.nout) return;
    const bool active = (k >= J.klo) && (k < J.khi);
    const double sc = (k == 0) ? J.s0 : ((k == J.N - 1) ? J.sl : J.sm);
    const double y = active ? v * sc * J.gscale : 0.0;
    out[(long long)k * J.out_sk] = y;
    if (J.epi) acc_epilogue(b.acc, (long long)line * J.out_sl + (long long)k * J.out_sk, y);
  };
  auto step = [&](int& m, int inc) {
    m += inc;
    if (m >= D4) m -= D4;
  };
  int m[kYR], inc[kYR];
  const int a0 = max(J.jlo, 1);
#pragma unroll
  for (int r = 0; r < kYR; ++r) {
    const int kk = J.ak * (k0 + r) + J.bk;
    inc[r] = mod4d((long long)J.aj * kk, D4);
    m[r] = mod4d((long long)(J.aj * a0 + J.bj) * kk + J.off, D4);
  }
  if (J.mode == 1 && J.ty) {
    // twiddle rows: row j, columns k0 .. k0 + kYR - 1
    const double* __restrict__ T = J.ty + k0;
    const long long ld = J.ldy;
    double E[kYR], O[kYR], t[kYR];
#pragma unroll
    for (int r = 0; r < kYR; ++r) E[r] = O[r] = 0.0;
    const int a1 = min(j_end, J.N - 1);
    int j = a0;
    if (j < a1 && (j & 1)) {
      const double v = X(j);
      row8(T + j * ld, t);
#pragma unroll
      for (int r = 0; r < kYR; ++r) O[r] = fma(v, t[r], O[r]);
      ++j;
    }
    for (; j + 1 < a1; j += 2) {
      const double v0 = X(j), v1 = X(j + 1);
      double t1[kYR];
      row8(T + j * ld, t);
      row8(T + (j + 1) * ld, t1);
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        E[r] = fma(v0, t[r], E[r]);
        O[r] = fma(v1, t1[r], O[r]);
      }
    }
    if (j < a1) {
      const double v = X(j);
      row8(T + j * ld, t);
#pragma unroll
      for (int r = 0; r < kYR; ++r) E[r] = fma(v, t[r], E[r]);
    }
    double t0[kYR], tD[kYR];
    row8(T, t0);
    row8(T + D * ld, tD);
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      const int k = k0 + r;
      if (k >= J.nlane) break;
      double e = J.wm * E[r], o = J.wm * O[r];
      if (J.jlo == 0 && 0 < j_end) e = fma(J.w0 * X(0), t0[r], e);
      if (D >= J.jlo && D < j_end) {
        const double tt = J.wl * X(D) * tD[r];
        if (D & 1) o += tt;
        else e += tt;
      }
      put(k, e + o);
      if (D - k != k) put(D - k, is_sin ? o - e : e - o);
    }
  } else if (J.mode == 2 && J.ty) {
    const double* __restrict__ T = J.ty + k0;
    const long long ld = J.ldy;
    double acc[kYR], t[kYR];
#pragma unroll
    for (int r = 0; r < kYR; ++r) acc[r] = 0.0;
    const int pe = (D + 1) / 2;  // interior pairs j < D - j
    for (int j = 1; j < pe; ++j) {
      const double xa = X(j), xb = X(D - j);
      const double u = xa + xb, v = xa - xb;
      row8(T + j * ld, t);
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        const bool use_v = (((k0 + r) & 1) == 0) != !is_sin;
        acc[r] = fma(use_v ? v : u, t[r], acc[r]);
      }
    }
    double t0[kYR], tm[kYR];
    row8(T, t0);
    row8(T + (D / 2) * ld, tm);
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      const int k = k0 + r;
      if (k >= J.nlane) break;
      double tt = J.wm * acc[r];
      if (J.jlo == 0) {
        const double xa = X(0), xb = X(D);
        tt = fma(J.w0 * (((k & 1) == 0) ? xa + xb : xa - xb), t0[r], tt);
      }
      if ((D & 1) == 0) {
        const int jm = D / 2;
        if (jm >= J.jlo && jm < J.jhi) tt = fma(J.wm * X(jm), tm[r], tt);
      }
      put(k, tt);
    }
  } else if (J.mode == 1) {
    double E[kYR], O[kYR];
#pragma unroll
    for (int r = 0; r < kYR; ++r) E[r] = O[r] = 0.0;
    const int a1 = min(j_end, J.N - 1);
    int j = a0;
    if (j < a1 && (j & 1)) {
      const double v = X(j);
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        O[r] = fma(v, twiddle(J.q, D, m[r]), O[r]);
        step(m[r], inc[r]);
      }
      ++j;
    }
    for (; j + 1 < a1; j += 2) {
      const double v0 = X(j), v1 = X(j + 1);
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        E[r] = fma(v0, twiddle(J.q, D, m[r]), E[r]);
        step(m[r], inc[r]);
        O[r] = fma(v1, twiddle(J.q, D, m[r]), O[r]);
        step(m[r], inc[r]);
      }
    }
    if (j < a1) {
      const double v = X(j);
#pragma unroll
      for (int r = 0; r < kYR; ++r) E[r] = fma(v, twiddle(J.q, D, m[r]), E[r]);
    }
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      const int k = k0 + r;
      if (k >= J.nlane) break;
      double e = J.wm * E[r], o = J.wm * O[r];
      if (J.jlo == 0 && 0 < j_end) e = fma(J.w0 * X(0), twiddle(J.q, D, mod4d(J.off, D4)), e);
      if (D >= J.jlo && D < j_end) {
        const double t = J.wl * X(D) *
                         twiddle(J.q, D, mod4d((long long)2 * D * k + J.off, D4));
        if (D & 1) o += t;
        else e += t;
      }
      put(k, e + o);
      if (D - k != k) put(D - k, is_sin ? o - e : e - o);
    }
  } else if (J.mode == 2) {
    double acc[kYR];
#pragma unroll
    for (int r = 0; r < kYR; ++r) acc[r] = 0.0;
    // cos: even k pairs with u; sin: even k pairs with v
    const int pe = (D + 1) / 2;  // interior pairs j < D - j
    for (int j = 1; j < pe; ++j) {
      const double xa = X(j), xb = X(D - j);
      const double u = xa + xb, v = xa - xb;
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        const bool use_v = (((k0 + r) & 1) == 0) != !is_sin;
        acc[r] = fma(use_v ? v : u, twiddle(J.q, D, m[r]), acc[r]);
        step(m[r], inc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      const int k = k0 + r;
      if (k >= J.nlane) break;
      double t = J.wm * acc[r];
      if (J.jlo == 0) {  // the end pair (0, D) with the end weight
        const double xa = X(0), xb = X(D);
        t = fma(J.w0 * (((k & 1) == 0) ? xa + xb : xa - xb), twiddle(J.q, D, mod4d(J.off, D4)), t);
      }
      if ((D & 1) == 0) {
        const int jm = D / 2;
        if (jm >= J.jlo && jm < J.jhi)
          t = fma(J.wm * X(jm),
                  twiddle(J.q, D, mod4d((long long)2 * jm * k + J.off, D4)), t);
      }
      put(k, t);
    }
  } else {
    double acc[kYR];
#pragma unroll
    for (int r = 0; r < kYR; ++r) acc[r] = 0.0;
    const int a1 = min(j_end, J.N - 1);
    for (int j = a0; j < a1; ++j) {
      const double v = X(j);
#pragma unroll
      for (int r = 0; r < kYR; ++r) {
        acc[r] = fma(v, twiddle(J.q, D, m[r]), acc[r]);
        step(m[r], inc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      const int k = k0 + r;
      if (k >= J.nout) break;
      double t = J.wm * acc[r];
      const int kk = J.ak * k + J.bk;
      if (J.jlo == 0 && 0 < j_end) {
        const int mm = mod4d((long long)J.bj * kk + J.off, D4);
        t = fma(J.w0 * X(0), twiddle(J.q, D, mm), t);
      }
      const int jl = J.N - 1;
      if (jl > 0 && jl >= J.jlo && jl < j_end) {
        const int mm = mod4d((long long)(J.aj * jl + J.bj) * kk + J.off, D4);
        t = fma(J.wl * X(jl), twiddle(J.q, D, mm), t);
      }
      put(k, t);
    }
  }
}

// Two-level passes for REDFT00 / RODFT00 kinds when D = A * B.  With
// j = B j1 + j2, pi j k / D = pi j1 k / A + pi j2 k / D, so
//   cos-kind: y_k = sum_j2 [cos(pi j2 k/D) C(j2,k) - sin(pi j2 k/D) S(j2,k)]
//   sin-kind: y_k = sum_j2 [cos(pi j2 k/D) S(j2,k) + sin(pi j2 k/D) C(j2,k)]
// with C, S = sum_j1 w_j x_j cos / sin(pi j1 k / A), which depend on k only
// through k mod 2A (C even, S odd about A).  Pass 1 computes C, S for
// k' = 0..A; pass 2 combines them.  Work: about (A+2) nin + 2 B nout FMAs
// (B nout when outputs pair up, see pass 2) instead of about nin * nout / 2
// for the direct sum.
//
// Both passes first issue all of their global loads (inputs, partial sums
// and twiddles staged in shared memory), then run FMA loops over shared
// memory: one round trip to L2 per pass instead of a chain of dependent
// scattered loads.
constexpr int kP1Threads = 128;
constexpr int kP2Threads = 128;  // 4 warps split the j2 sum of 32 outputs
constexpr int kP2Warps = kP2Threads / 32;

// Thread-block clusters: a sum too long for one SM is split over the CTAs of
// a cluster, whose partial results are combined through distributed shared
// memory by rank 0 in rank order.
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" :::
                   "memory");
}
__device__ __forceinline__ double ld_cluster(const double* local, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned ra;
  double v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
  return v;
}

// pass 1: cluster = (job, line, group of kpc consecutive k' <= A/2); CTA r
// of the cluster sums j1 in its slice of [0, K).  The even and odd j1 terms
// are summed apart: cos / sin(pi j1 (A - k') / A) = +-(-1)^j1 cos / sin(pi
// j1 k' / A), so the same four sums give C, S at k' and at A - k' and half
// of the k' are computed.  Threads own (k', part, j2) items with j2
// fastest: staged inputs are read without bank conflicts and the j1
// twiddles are broadcast.  Slices hold an even number of j1 (Kc2), so a
// local index has the parity of its global j1.
__host__ __device__ inline int p1_half(int A) { return A / 2; }
__host__ __device__ inline int p1_slice(int K, int ncl) { return (((K + ncl - 1) / ncl) + 1) & ~1; }

template <int NJ>
__global__ void __launch_bounds__(kP1Threads) two_level_pass1(const AxisBatchT<NJ> b, int kpc, int ncl) {
  extern __shared__ double sm1[];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D4 = 4 * D, H = p1_half(A);
  const int ngrp = (H + 1 + kpc - 1) / kpc;
  const int local = (blockIdx.x - b.start[jb]) / ncl;
  const unsigned rank = ncl > 1 ? cluster_rank() : 0u;
  const int line = local / ngrp;
  const int kp0 = (local - line * ngrp) * kpc;
  const int nkp = min(kpc, H + 1 - kp0);
  const int j_end = min(J.jhi, J.nin);  // terms j in [jlo, j_end)
  const int K = (j_end + B - 1) / B;
  const int Kc = p1_slice(K, ncl);
  const int ja1 = min(K, (int)rank * Kc), Kl = min(K, ja1 + Kc) - ja1;
  const int Klp = (Kl + 1) & ~1;    // padded to whole (even, odd) pairs
  double* fin = sm1;                // kpc * B (C, S, C', S') of this CTA's slice
  double* xs = fin + 4 * kpc * B;   // Kc * B weighted inputs, zero outside the sum
  double* tc = xs + Kc * B;         // kpc * Kc cos(pi j1 k' / A)
  double* ts = tc + kpc * Kc;       // kpc * Kc sin(pi j1 k' / A)
  double* red = ts + kpc * Kc;      // partial sums of the items
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const double* __restrict__ wr = J.win ? J.win + (long long)line * J.win_sl : nullptr;
  auto stage_twiddles = [&]() {
    for (int t = threadIdx.x; t < nkp * Klp; t += kP1Threads) {
      const int kpl = t / Klp, jl = t - kpl * Klp;
      double c = 0.0, sn = 0.0;
      if (jl < Kl) {
        // pi j1 k' / A = pi (2 B j1 k') / (2 D); both factors below 4D
        const unsigned step = (2u * (unsigned)B * (unsigned)(kp0 + kpl)) % (unsigned)D4;
        const int m = (int)((step * (unsigned)(ja1 + jl)) % (unsigned)D4);
        c = twiddle(J.q, D, m);
        sn = twiddle(J.q, D, m >= D ? m - D : m + 3 * D);
      }
      tc[kpl * Kc + jl] = c;
      ts[kpl * Kc + jl] = sn;
    }
  };
  if (b.early) stage_twiddles();
  pdl_wait();
  if (!b.early) stage_twiddles();
  for (int t = threadIdx.x; t < Klp * B; t += kP1Threads) {
    const int j = ja1 * B + t;
    double v = 0.0;
    if (t < Kl * B && j >= J.jlo && j < j_end) {
      const double w = (j == 0) ? J.w0 : ((j == J.N - 1) ? J.wl : J.wm);
      v = w * in_at(x, J.in_sk, wr, J.win_sk, j);
    }
    xs[t] = v;
  }
  __syncthreads();
  const int P = max(1, kP1Threads / (nkp * B));  // parts splitting the j1 pair sum
  const int nitem = nkp * P * B;
  const int npair = Klp / 2;
  for (int it = threadIdx.x; it < nitem; it += kP1Threads) {
    const int j2 = it % B, r = it / B;
    const int part = r % P, kpl = r / P;
    const double* tcp = tc + kpl * Kc;
    const double* tsp = ts + kpl * Kc;
    double ce = 0.0, se = 0.0, co = 0.0, so = 0.0;
#pragma unroll 2
    for (int q = part; q < npair; q += P) {
      const double v0 = xs[(2 * q) * B + j2], v1 = xs[(2 * q + 1) * B + j2];
      ce = fma(v0, tcp[2 * q], ce);
      se = fma(v0, tsp[2 * q], se);
      co = fma(v1, tcp[2 * q + 1], co);
      so = fma(v1, tsp[2 * q + 1], so);
    }
    red[4 * it] = ce + co;      // C(k')
    red[4 * it + 1] = se + so;  // S(k')
    red[4 * it + 2] = ce - co;  // C(A - k')
    red[4 * it + 3] = so - se;  // S(A - k')
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nkp * B; t += kP1Threads) {
    const int j2 = t % B, kpl = t / B;
    double f[4] = {0.0, 0.0, 0.0, 0.0};
    for (int part = 0; part < P; ++part) {
      const int it = (kpl * P + part) * B + j2;
#pragma unroll
      for (int u = 0; u < 4; ++u) f[u] += red[4 * it + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) fin[4 * t + u] = f[u];
  }
  if (ncl > 1) cluster_sync_all();
  else __syncthreads();
  if (rank == 0) {
    for (int t = threadIdx.x; t < nkp * B; t += kP1Threads) {
      double f[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) f[u] = fin[4 * t + u];
      for (int r = 1; r < ncl; ++r)
#pragma unroll
        for (int u = 0; u < 4; ++u) f[u] += ld_cluster(fin + 4 * t + u, (unsigned)r);
      const int j2 = t % B, kp = kp0 + t / B;
      double* cs = J.cs + (((long long)line * B + j2) * (A + 1)) * 2;
      cs[2 * kp] = f[0];
      cs[2 * kp + 1] = f[1];
      if (A - kp != kp) {
        cs[2 * (A - kp)] = f[2];
        cs[2 * (A - kp) + 1] = f[3];
      }
    }
  }
  if (ncl > 1) cluster_sync_all();  // remote reads done before any CTA exits
}

// pass 2: cluster = (job, line, 32 outputs); CTA r of the cluster sums j2 in
// its slice of [0, B).  The slice's twiddles cos/sin(pi j2 k / D) are staged
// first; lanes own outputs (their C, S loads are contiguous), warps split
// the slice and are combined in a fixed order.
//
// Paired jobs (mode 1: B even, every output wanted): with B even, (-1)^j =
// (-1)^j2, so y(D - k) = +-sum_j2 (-1)^j2 T_j2(k) for the terms T_j2(k) of
// y(k).  Lanes own k <= D/2; warps (and cluster slices, of even length)
// hold j2 of one parity, and the even and odd sums E, O give y(k) = E + O
// and y(D - k) = E - O (cos kind) or O - E (sin kind).
__host__ __device__ inline int p2_slice(int B, int ncl, bool paired) {
  const int c = (B + ncl - 1) / ncl;
  return (paired && ncl > 1) ? ((c + 1) & ~1) : c;
}
__host__ __device__ inline int p2_lanes(const AxisJob& J) { return J.mode == 1 ? J.D / 2 + 1 : J.nout; }

__device__ __forceinline__ void p2_put(const AxisJob& J, const AccEpi& acc, int line, int k, double y) {
  if (k >= J.nout) return;
  const bool on = k >= J.klo && k < J.khi;
  const long long e = (long long)line * J.out_sl + (long long)k * J.out_sk;
  const double sc = (k == 0) ? J.s0 : ((k == J.N - 1) ? J.sl : J.sm);
  const double v = on ? y * sc * J.gscale : 0.0;
  J.out[e] = v;
  if (J.epi) acc_epilogue(acc, e, v);
}

template <int NJ>
__global__ void __launch_bounds__(kP2Threads) two_level_pass2(const AxisBatchT<NJ> b, int ncl) {
  extern __shared__ double sm2[];
  __shared__ double red[kP2Warps][32];
  __shared__ double fin[2][32];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D4 = 4 * D;
  const bool paired = J.mode == 1;
  const int nlane = p2_lanes(J);
  const int nkb = (nlane + 31) / 32;
  const int local = (blockIdx.x - b.start[jb]) / ncl;
  const unsigned rank = ncl > 1 ? cluster_rank() : 0u;
  const int line = local / nkb;
  const int k0 = (local - line * nkb) * 32;
  const int Bc = p2_slice(B, ncl, paired);
  const int ja2 = min(B, (int)rank * Bc), Bl = min(B, ja2 + Bc) - ja2;
  auto stage_twiddles = [&]() {
    for (int t = threadIdx.x; t < Bl * 32; t += kP2Threads) {
      const int j2 = ja2 + (t >> 5), k = k0 + (t & 31);
      // pi j2 k / D; j2 < D and k < N, so 2 j2 k fits in 32 bits for N < 32768
      const int m = (int)((2u * (unsigned)j2 * (unsigned)k) % (unsigned)D4);
      sm2[2 * t] = twiddle(J.q, D, m);
      sm2[2 * t + 1] = twiddle(J.q, D, m >= D ? m - D : m + 3 * D);
    }
  };
  if (b.early) stage_twiddles();
  pdl_wait();
  if (!b.early) stage_twiddles();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = k0 + lane;
  const bool on = paired ? k < nlane : (k < J.nout && k >= J.klo && k < J.khi);
  int kp = k % (2 * A);
  double ssign = 1.0;
  if (kp > A) {
    kp = 2 * A - kp;
    ssign = -1.0;
  }
  const bool is_sin = (J.off != 0);
  const double* cs = J.cs + ((long long)line * B * (A + 1) + kp) * 2;
  // C, S of this lane's j2 terms, loaded before the twiddles are needed
  constexpr int kMaxOwn = 16;
  double Cv[kMaxOwn], Sv[kMaxOwn];
  const int nown = on ? min(kMaxOwn, (Bl - warp + kP2Warps - 1) / kP2Warps) : 0;
#pragma unroll
  for (int i = 0; i < kMaxOwn; ++i) {
    if (i < nown) {
      const long long o = (long long)(ja2 + warp + i * kP2Warps) * (A + 1) * 2;
      Cv[i] = __ldcg(cs + o);
      Sv[i] = __ldcg(cs + o + 1);
    }
  }
  __syncthreads();
  double acc = 0.0;
#pragma unroll
  for (int i = 0; i < kMaxOwn; ++i) {
    if (i < nown) {
      const int t = warp + i * kP2Warps;  // j2 - ja2
      const double cw = sm2[2 * (t * 32 + lane)], sw = sm2[2 * (t * 32 + lane) + 1];
      const double S = ssign * Sv[i];
      if (is_sin) acc = fma(cw, S, fma(sw, Cv[i], acc));
      else acc = fma(cw, Cv[i], fma(-sw, S, acc));
    }
  }
  // j2 beyond the register-held terms
  if (on) {
    for (int t = warp + kMaxOwn * kP2Warps; t < Bl; t += kP2Warps) {
      const long long o = (long long)(ja2 + t) * (A + 1) * 2;
      const double cw = sm2[2 * (t * 32 + lane)], sw = sm2[2 * (t * 32 + lane) + 1];
      const double C = __ldcg(cs + o), S = ssign * __ldcg(cs + o + 1);
      if (is_sin) acc = fma(cw, S, fma(sw, C, acc));
      else acc = fma(cw, C, fma(-sw, S, acc));
    }
  }
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0) {
    if (paired) {
      // warps of even index hold even j2 (kP2Warps and ja2 are even)
      double e = 0.0, o = 0.0;
#pragma unroll
      for (int w = 0; w < kP2Warps; w += 2) {
        e += red[w][lane];
        o += red[w + 1][lane];
      }
      fin[0][lane] = e;
      fin[1][lane] = o;
    } else {
      double y = 0.0;
#pragma unroll
      for (int w = 0; w < kP2Warps; ++w) y += red[w][lane];
      fin[0][lane] = y;
    }
  }
  if (ncl > 1) cluster_sync_all();
  else __syncthreads();
  if (rank == 0 && warp == 0) {
    double y = fin[0][lane];
    for (int r = 1; r < ncl; ++r) y += ld_cluster(&fin[0][lane], (unsigned)r);
    if (paired) {
      double o = fin[1][lane];
      for (int r = 1; r < ncl; ++r) o += ld_cluster(&fin[1][lane], (unsigned)r);
      if (k < nlane) {
        p2_put(J, b.acc, line, k, y + o);
        if (D - k != k) p2_put(J, b.acc, line, D - k, is_sin ? o - y : y - o);
      }
    } else if (k < J.nout) {
      p2_put(J, b.acc, line, k, on ? y : 0.0);
    }
  }
  if (ncl > 1) cluster_sync_all();  // remote reads done before any CTA exits
}

// pass 2 for launches with many lines (the x passes of 3-D tanks):
// CTA = (job, 32 outputs, group of lpc lines).  The B x 32 twiddle tile is
// staged once for the group; each warp takes lines in turn and sums all of
// their j2 terms, so no cross-warp reduction is needed.
template <int NJ>
__global__ void __launch_bounds__(kP2Threads) two_level_pass2_lines(const AxisBatchT<NJ> b, int lpc) {
  extern __shared__ double sm2[];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D4 = 4 * D;
  const bool paired = J.mode == 1;
  const int nlane = p2_lanes(J);
  const int nkb = (nlane + 31) / 32;
  const int local = blockIdx.x - b.start[jb];
  const int kb = local % nkb;
  const int l0 = (local / nkb) * lpc;
  const int k0 = kb * 32;
  auto stage_twiddles = [&]() {
    for (int t = threadIdx.x; t < B * 32; t += kP2Threads) {
      const int j2 = t >> 5, k = k0 + (t & 31);
      const int m = (int)((2u * (unsigned)j2 * (unsigned)k) % (unsigned)D4);
      sm2[2 * t] = twiddle(J.q, D, m);
      sm2[2 * t + 1] = twiddle(J.q, D, m >= D ? m - D : m + 3 * D);
    }
  };
  if (b.early) stage_twiddles();
  pdl_wait();
  if (!b.early) stage_twiddles();
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = k0 + lane;
  const bool on = paired ? k < nlane : (k < J.nout && k >= J.klo && k < J.khi);
  int kp = k % (2 * A);
  double ssign = 1.0;
  if (kp > A) {
    kp = 2 * A - kp;
    ssign = -1.0;
  }
  const bool is_sin = (J.off != 0);
  const double2* tw = reinterpret_cast<const double2*>(sm2) + lane;
  const int l1 = min(J.nlines, l0 + lpc);
  for (int line = l0 + warp; line < l1; line += kP2Warps) {
    const double* cs = J.cs + ((long long)line * B * (A + 1) + kp) * 2;
    double ae = 0.0, ao = 0.0;  // even, odd j2 (paired jobs; else all in ae)
    if (on) {
#pragma unroll 4
      for (int j2 = 0; j2 < B; ++j2) {
        const long long o = (long long)j2 * (A + 1) * 2;
        const double C = __ldcg(cs + o), S = ssign * __ldcg(cs + o + 1);
        const double2 t = tw[j2 * 32];
        if (paired && (j2 & 1)) {  // j2 is warp-uniform
          if (is_sin) ao = fma(t.x, S, fma(t.y, C, ao));
          else ao = fma(t.x, C, fma(-t.y, S, ao));
        } else {
          if (is_sin) ae = fma(t.x, S, fma(t.y, C, ae));
          else ae = fma(t.x, C, fma(-t.y, S, ae));
        }
      }
    }
    if (paired) {
      if (k < nlane) {
        p2_put(J, b.acc, line, k, ae + ao);
        if (D - k != k) p2_put(J, b.acc, line, D - k, is_sin ? ao - ae : ae - ao);
      }
    } else {
      p2_put(J, b.acc, line, k, on ? ae : 0.0);
    }
  }
}

// Fused two-level pass for launches with few lines (the x passes of 2-D
// tanks).  The outputs k whose folded class k' (k mod 2A, reflected about
// A) is g or A - g need the pass-1 values C, S at those two k' only, and
// pass 1 gives both from one even/odd j1 sum.  So one CTA per (job, line,
// class pair g <= A/2, output split u) computes C, S of its pair into
// shared memory and then the outputs of its pair: both passes in one
// launch, no partial sums through global memory, and no communication
// between CTAs.  A half-period cos table is staged whole in shared memory
// (before griddepcontrol.wait when it is constant).  With nsplit > 1 the
// outputs of a pair are dealt round-robin to nsplit CTAs, each of which
// repeats the (short) pass 1.
constexpr int kFThreads = 256;
constexpr int kFWarps = kFThreads / 32;

// distinct residues k mod 2A of class pair g, ascending: {g, A-g, A+g, 2A-g}
__host__ __device__ inline int fused_residues(int A, int g, int* r) {
  if (g == 0) { r[0] = 0; r[1] = A; return 2; }
  if (2 * g == A) { r[0] = g; r[1] = A + g; return 2; }
  r[0] = g; r[1] = A - g; r[2] = A + g; r[3] = 2 * A - g;
  return 4;
}
// residue i of fused_residues(A, g, .), without an indexed local array
__host__ __device__ inline int fused_residue(int A, int g, int i) {
  if (g == 0) return i == 0 ? 0 : A;
  if (2 * g == A) return i == 0 ? g : A + g;
  return i == 0 ? g : (i == 1 ? A - g : (i == 2 ? A + g : 2 * A - g));
}
// number of outputs k < nlane in class pair g
__host__ __device__ inline int fused_slots(int A, int g, int nlane) {
  int r[4];
  const int nr = fused_residues(A, g, r);
  const int per = nlane / (2 * A), rem = nlane - per * 2 * A;
  int n = per * nr;
  for (int i = 0; i < nr; ++i) n += r[i] < rem ? 1 : 0;
  return n;
}
// j2 parts of pass 2 for nsb blocks of 32 outputs (even: parts keep the
// parity of j2, which paired outputs need)
__host__ __device__ inline int fused_parts(int nsb) {
  if (nsb <= 0 || nsb >= kFWarps) return 2;
  const int p = (kFWarps / nsb) & ~1;
  return p < 2 ? 2 : p;
}
__host__ __device__ inline int fused_p1_parts(int B) { return B >= kFThreads ? 1 : kFThreads / B; }

template <int NJ>
__global__ void __launch_bounds__(kFThreads) two_level_fused(const AxisBatchT<NJ> b, int nsplit) {
  extern __shared__ double smf[];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D2 = 2 * D, D4 = 4 * D, H = A / 2;
  const int local = blockIdx.x - b.start[jb];
  const int line = local / ((H + 1) * nsplit);
  const int rem = local - line * (H + 1) * nsplit;
  const int g = rem / nsplit, u = rem - g * nsplit;
  const bool paired = J.mode == 1;
  const bool is_sin = (J.off != 0);
  const int nlane = paired ? D / 2 + 1 : J.nout;
  const int j_end = min(J.jhi, J.nin);
  const int K = (j_end + B - 1) / B;
  const int Klp = (K + 1) & ~1;
  // FP64 work on this GPU is scarce (about 2 operations per clock per SM),
  // so the inner loops issue FMAs only: the table covers a half period, so
  // a lookup needs no sign change, and signs and weights are applied to
  // the few sums, not to the terms.
  double* qh = smf;                 // 2D + 1: cos(pi m / (2D)), m = 0..2D
  double* xs = qh + (D2 + 1);       // Klp * B inputs, zero outside the sum
  double* csm = xs + Klp * B;       // B x {C(g), S(g), C(A-g), S(A-g)}
  double* red = csm + 4 * B;        // partial sums of both passes
  auto stage_table = [&]() {
    // cos(pi m/(2D)) = -cos(pi (2D - m)/(2D)): the sign bit is flipped as an
    // integer
    for (int t = threadIdx.x; t <= D2; t += kFThreads)
      qh[t] = t <= D ? __ldg(J.q + t)
                     : __longlong_as_double(__double_as_longlong(__ldg(J.q + (D2 - t))) ^ (1LL << 63));
  };
  auto cosm = [&](int m) { return qh[m <= D2 ? m : D4 - m]; };                 // m in [0, 4D)
  auto sinm = [&](int m) { return cosm(m >= D ? m - D : m + 3 * D); };
  if (b.early) stage_table();
  pdl_wait();
  if (!b.early) stage_table();
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const double* __restrict__ wr = J.win ? J.win + (long long)line * J.win_sl : nullptr;
  // interior inputs enter with weight wm, applied to the sums below; the two
  // end points carry w0 / wm and wl / wm
  const double e0 = J.w0 / J.wm, el = J.wl / J.wm;
  for (int t = threadIdx.x; t < Klp * B; t += kFThreads) {
    double v = 0.0;
    if (t >= J.jlo && t < j_end) {
      v = wr ? __ldg(x + (long long)t * J.in_sk) * __ldg(wr + (long long)t * J.win_sk)
             : __ldg(x + (long long)t * J.in_sk);
      if (t == 0) v *= e0;
      else if (t == J.N - 1) v *= el;
    }
    xs[t] = v;
  }
  __syncthreads();
  // pass 1: items (j2, part); part sums the j1 pairs q = part, part + P1, ...
  const int P1 = fused_p1_parts(B);
  const int npair = Klp / 2;
  {
    const int stp = (int)((2LL * B * g) % D4);                      // angle index of j1 = 1
    const int inc = (int)((2LL * stp * (long long)P1) % D4);        // j1 -> j1 + 2 P1
    for (int it = threadIdx.x; it < P1 * B; it += kFThreads) {
      const int j2 = it % B, part = it / B;
      double ce = 0.0, se = 0.0, co = 0.0, so = 0.0;
      int m = (int)((2LL * stp * (long long)part) % D4);           // j1 = 2 part
      for (int q = part; q < npair; q += P1) {
        int m1 = m + stp;
        if (m1 >= D4) m1 -= D4;
        const double v0 = xs[(2 * q) * B + j2], v1 = xs[(2 * q + 1) * B + j2];
        ce = fma(v0, cosm(m), ce);
        se = fma(v0, sinm(m), se);
        co = fma(v1, cosm(m1), co);
        so = fma(v1, sinm(m1), so);
        m += inc;
        if (m >= D4) m -= D4;
      }
      red[4 * it] = ce + co;      // C(g)
      red[4 * it + 1] = se + so;  // S(g)
      red[4 * it + 2] = ce - co;  // C(A - g)
      red[4 * it + 3] = so - se;  // S(A - g)
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < B; t += kFThreads) {
    double f[4] = {0.0, 0.0, 0.0, 0.0};
    for (int part = 0; part < P1; ++part)
#pragma unroll
      for (int v = 0; v < 4; ++v) f[v] += red[4 * (part * B + t) + v];
#pragma unroll
    for (int v = 0; v < 4; ++v) csm[4 * t + v] = f[v] * J.wm;
  }
  __syncthreads();
  // pass 2: this CTA's outputs are the slots s = t nsplit + u of the pair
  const int nr = (g == 0 || 2 * g == A) ? 2 : 4;
  const int nslot = fused_slots(A, g, nlane);
  const int nu = nslot > u ? (nslot - u + nsplit - 1) / nsplit : 0;
  const int nsb = (nu + 31) / 32;
  const int P = fused_parts(nsb);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int item = warp; item < nsb * P; item += kFWarps) {
    const int sb = item / P, p = item - sb * P;
    const int t = sb * 32 + lane;
    double y = 0.0;
    if (t < nu) {
      const int s = t * nsplit + u;
      const int k = 2 * A * (s / nr) + fused_residue(A, g, s % nr);
      int kp = k % (2 * A);
      double ssign = 1.0;
      if (kp > A) { kp = 2 * A - kp; ssign = -1.0; }
      const double* cp = csm + (kp == g ? 0 : 2);
      int m = (int)((2LL * p * k) % D4);
      const int inc = (int)((2LL * P * k) % D4);
      // cos kind: y = sum cw C - ssign sum sw S; sin kind: y = ssign sum cw S + sum sw C
      double a1 = 0.0, a2 = 0.0;
      if (is_sin) {
        for (int j2 = p; j2 < B; j2 += P) {
          a1 = fma(cosm(m), cp[4 * j2 + 1], a1);
          a2 = fma(sinm(m), cp[4 * j2], a2);
          m += inc;
          if (m >= D4) m -= D4;
        }
        y = fma(ssign, a1, a2);
      } else {
        for (int j2 = p; j2 < B; j2 += P) {
          a1 = fma(cosm(m), cp[4 * j2], a1);
          a2 = fma(sinm(m), cp[4 * j2 + 1], a2);
          m += inc;
          if (m >= D4) m -= D4;
        }
        y = fma(-ssign, a2, a1);
      }
    }
    red[item * 32 + lane] = y;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nu; t += kFThreads) {
    const int sb = t >> 5, ln = t & 31;
    double e = 0.0, o = 0.0;
    for (int p = 0; p < P; p += 2) {
      e += red[(sb * P + p) * 32 + ln];
      o += red[(sb * P + p + 1) * 32 + ln];
    }
    const int s = t * nsplit + u;
    const int k = 2 * A * (s / nr) + fused_residue(A, g, s % nr);
    if (paired) {
      p2_put(J, b.acc, line, k, e + o);
      if (D - k != k) p2_put(J, b.acc, line, D - k, is_sin ? o - e : e - o);
    } else {
      p2_put(J, b.acc, line, k, e + o);
    }
  }
}

// Two-level y passes (REDFT00 / RODFT00 along a strided axis, lines
// contiguous): the same split as above, with lanes owning lines so that
// every load and store is coalesced and every twiddle is warp-uniform.
// The partial sums are stored [((j2 (A+1) + k') 2 + {C, S}) nlines + line].
constexpr int kYT = 128;   // lines per CTA
constexpr int kYKF = 9;    // k' <= A/2 per pass-1 CTA (four accumulators each)
constexpr int kYQ = 20;    // outputs of one k' class per pass-2 thread
constexpr int kYH = 12;    // outputs k <= D/2 of one class per thread (paired jobs)

// pass 1: CTA = (job, k' chunk, j2, block of kYT lines).  As in the x pass,
// the even and odd j1 terms are summed apart, which gives C, S at k' and at
// A - k' from the same sums: only k' <= A/2 are computed.
template <int NJ>
__global__ void __launch_bounds__(kYT) ytl_pass1(const AxisBatchT<NJ> b) {
  extern __shared__ double smy[];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D4 = 4 * D, H = A / 2;
  const int nkc = (H + 1 + kYKF - 1) / kYKF;
  int local = blockIdx.x - b.start[jb];
  const int kc = local % nkc;
  local /= nkc;
  const int j2 = local % B;
  const int lb = local / B;
  const int kp0 = kc * kYKF, nkp = min(kYKF, H + 1 - kp0);
  const int j_end = min(J.jhi, J.nin);
  const int K = (j_end + B - 1) / B;
  const int Kp = (K + 1) & ~1;    // whole (even, odd) pairs
  double* tc = smy;               // Kp x kYKF cos(pi j1 k' / A), zero beyond K
  double* ts = tc + Kp * kYKF;    // Kp x kYKF sin(pi j1 k' / A)
  auto stage = [&]() {
    for (int t = threadIdx.x; t < Kp * kYKF; t += kYT) {
      const int j1 = t / kYKF, kpl = t - j1 * kYKF;
      double c = 0.0, sn = 0.0;
      if (kpl < nkp && j1 < K) {
        const unsigned step = (2u * (unsigned)B * (unsigned)(kp0 + kpl)) % (unsigned)D4;
        const int m = (int)((step * (unsigned)j1) % (unsigned)D4);
        c = twiddle(J.q, D, m);
        sn = twiddle(J.q, D, m >= D ? m - D : m + 3 * D);
      }
      tc[t] = c;
      ts[t] = sn;
    }
  };
  if (b.early) stage();
  pdl_wait();
  if (!b.early) stage();
  __syncthreads();
  const int line = lb * kYT + threadIdx.x;
  if (line >= J.nlines) return;
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const double* __restrict__ wr = J.win ? J.win + (long long)line * J.win_sl : nullptr;
  double ce[kYKF], co[kYKF], se[kYKF], so[kYKF];
#pragma unroll
  for (int r = 0; r < kYKF; ++r) ce[r] = co[r] = se[r] = so[r] = 0.0;
  for (int j1 = 0; j1 < K; j1 += 2) {
    const int j = B * j1 + j2, jo = j + B;
    double v0 = 0.0, v1 = 0.0;
    if (j >= J.jlo && j < j_end) {
      const double w = (j == 0) ? J.w0 : ((j == J.N - 1) ? J.wl : J.wm);
      v0 = w * in_at(x, J.in_sk, wr, J.win_sk, j);
    }
    if (j1 + 1 < K && jo >= J.jlo && jo < j_end) {
      const double w = (jo == J.N - 1) ? J.wl : J.wm;
      v1 = w * in_at(x, J.in_sk, wr, J.win_sk, jo);
    }
    const double* t0 = tc + j1 * kYKF;
    const double* s0 = ts + j1 * kYKF;
#pragma unroll
    for (int r = 0; r < kYKF; ++r) {
      ce[r] = fma(v0, t0[r], ce[r]);
      se[r] = fma(v0, s0[r], se[r]);
      co[r] = fma(v1, t0[kYKF + r], co[r]);
      so[r] = fma(v1, s0[kYKF + r], so[r]);
    }
  }
  const long long nl = J.nlines;
  double* o = J.cs + (long long)j2 * (A + 1) * 2 * nl + line;
#pragma unroll
  for (int r = 0; r < kYKF; ++r) {
    if (r < nkp) {
      const int kp = kp0 + r;
      o[(2 * kp) * nl] = ce[r] + co[r];
      o[(2 * kp + 1) * nl] = se[r] + so[r];
      if (A - kp != kp) {
        o[(2 * (A - kp)) * nl] = ce[r] - co[r];
        o[(2 * (A - kp) + 1) * nl] = so[r] - se[r];
      }
    }
  }
}

// output o of class k': k = 2 A o + k' when k' is 0 or A, else alternately
// 2 A q + k' and 2 A (q + 1) - k' (folded, S enters with a minus sign)
__device__ __forceinline__ int ytl_k(int o, int A, int kp, bool pair) {
  if (!pair) return 2 * A * o + kp;
  const int q = o >> 1;
  return (o & 1) ? 2 * A * (q + 1) - kp : 2 * A * q + kp;
}

__device__ __forceinline__ void ytl_put(const AxisJob& J, const AccEpi& acc, int line, int k, double y) {
  if (k >= J.nout) return;
  const bool on = k >= J.klo && k < J.khi;
  const double sc = (k == 0) ? J.s0 : ((k == J.N - 1) ? J.sl : J.sm);
  const double v = on ? y * sc * J.gscale : 0.0;
  const long long e = (long long)line * J.out_sl + (long long)k * J.out_sk;
  J.out[e] = v;
  if (J.epi) acc_epilogue(acc, e, v);
}

// pass 2: CTA = (job, k', block of kYT lines); each C, S value is read once
// and feeds every output of its class.  Paired jobs (mode 1: B even, every
// output wanted): outputs k and D - k are in the same class, and with B
// even y(D - k) = +-sum_j2 (-1)^j2 T_j2(k); the thread sums even and odd j2
// apart for the class's outputs k <= D/2 and writes both.
template <int NJ>
__global__ void __launch_bounds__(kYT, 1) ytl_pass2(const AxisBatchT<NJ> b) {
  extern __shared__ double smy[];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int A = J.A, B = J.B, D = J.D, D4 = 4 * D;
  const int local = blockIdx.x - b.start[jb];
  const int kp = local % (A + 1);
  const int lb = local / (A + 1);
  const bool pair = kp > 0 && kp < A;
  const bool paired = J.mode == 1;
  double* tw = smy;  // B x kYQ (cos, sin)(pi j2 k / D)
  auto stage = [&]() {
    for (int t = threadIdx.x; t < B * kYQ; t += kYT) {
      const int j2 = t / kYQ, oi = t - j2 * kYQ;
      const int k = ytl_k(oi, A, kp, pair);
      double c = 0.0, sn = 0.0;
      if (k < J.nout) {
        const int m = (int)((2u * (unsigned)j2 * (unsigned)k) % (unsigned)D4);
        c = twiddle(J.q, D, m);
        sn = twiddle(J.q, D, m >= D ? m - D : m + 3 * D);
      }
      tw[2 * t] = c;
      tw[2 * t + 1] = sn;
    }
  };
  if (b.early) stage();
  pdl_wait();
  if (!b.early) stage();
  __syncthreads();
  const int line = lb * kYT + threadIdx.x;
  if (line >= J.nlines) return;
  const bool is_sin = (J.off != 0);
  const long long nl = J.nlines;
  const double* cs = J.cs + (long long)kp * 2 * nl + line;
  // outputs of this class below nout (uniform over the CTA)
  int nq = 0;
  while (nq < kYQ && ytl_k(nq, A, kp, pair) < J.nout) ++nq;
  if (paired) {
    int nc = 0;  // outputs k <= D/2 (the class's outputs increase with oi)
    while (nc < nq && nc < kYH && ytl_k(nc, A, kp, pair) <= D / 2) ++nc;
    double ae[kYH], ao[kYH];
#pragma unroll
    for (int oi = 0; oi < kYH; ++oi) ae[oi] = ao[oi] = 0.0;
    for (int j2 = 0; j2 < B; j2 += 2) {
      const long long base = (long long)j2 * (A + 1) * 2 * nl;
      const long long step = (long long)(A + 1) * 2 * nl;
      const double C0 = __ldcg(cs + base), S0 = __ldcg(cs + base + nl);
      const double C1 = __ldcg(cs + base + step), S1 = __ldcg(cs + base + step + nl);
      const double2* t0 = reinterpret_cast<const double2*>(tw) + j2 * kYQ;
      const double2* t1 = t0 + kYQ;
#pragma unroll
      for (int oi = 0; oi < kYH; ++oi) {
        if (oi < nc) {
          const bool neg = pair && (oi & 1);
          const double Sa = neg ? -S0 : S0, Sb = neg ? -S1 : S1;
          const double2 w0 = t0[oi], w1 = t1[oi];
          if (is_sin) {
            ae[oi] = fma(w0.x, Sa, fma(w0.y, C0, ae[oi]));
            ao[oi] = fma(w1.x, Sb, fma(w1.y, C1, ao[oi]));
          } else {
            ae[oi] = fma(w0.x, C0, fma(-w0.y, Sa, ae[oi]));
            ao[oi] = fma(w1.x, C1, fma(-w1.y, Sb, ao[oi]));
          }
        }
      }
    }
#pragma unroll
    for (int oi = 0; oi < kYH; ++oi) {
      if (oi < nc) {
        const int k = ytl_k(oi, A, kp, pair);
        ytl_put(J, b.acc, line, k, ae[oi] + ao[oi]);
        if (D - k != k) ytl_put(J, b.acc, line, D - k, is_sin ? ao[oi] - ae[oi] : ae[oi] - ao[oi]);
      }
    }
    return;
  }
  double acc[kYQ];
#pragma unroll
  for (int oi = 0; oi < kYQ; ++oi) acc[oi] = 0.0;
#pragma unroll 2
  for (int j2 = 0; j2 < B; ++j2) {
    const long long base = (long long)j2 * (A + 1) * 2 * nl;
    const double C = __ldcg(cs + base), S = __ldcg(cs + base + nl);
    const double2* t = reinterpret_cast<const double2*>(tw) + j2 * kYQ;
#pragma unroll
    for (int oi = 0; oi < kYQ; ++oi) {
      if (oi < nq) {
        const double Ss = (pair && (oi & 1)) ? -S : S;
        const double2 w = t[oi];
        acc[oi] = is_sin ? fma(w.x, Ss, fma(w.y, C, acc[oi])) : fma(w.x, C, fma(-w.y, Ss, acc[oi]));
      }
    }
  }
#pragma unroll
  for (int oi = 0; oi < kYQ; ++oi) {
    const int k = ytl_k(oi, A, kp, pair);
    if (oi < nq) ytl_put(J, b.acc, line, k, acc[oi]);
  }
}

// Fill the kind-dependent parameters of a pass.
void set_kind(AxisJob& J, int kind, int N, const double* q) {
  J.N = N;
  J.q = q;
  J.off = 0;
  J.jlo = 0;
  J.jhi = N;
  J.klo = 0;
  J.khi = N;
  J.w0 = J.wm = J.wl = 1.0;
  J.s0 = J.sm = J.sl = 1.0;
  switch (kind) {
    case K_C1_S2F:
    case K_C1_F2S:
    case K_S1_S2F:
    case K_S1_F2S: {
      const int D = N - 1;
      J.D = D;
      J.aj = 2; J.bj = 0; J.ak = 1; J.bk = 0;
      if (kind == K_C1_S2F) {
        J.w0 = 1.0; J.wm = 2.0; J.wl = 1.0;
        J.s0 = 1.0 / (2.0 * D); J.sm = 1.0 / D; J.sl = 1.0 / (2.0 * D);
      } else if (kind == K_S1_S2F || kind == K_S1_F2S) {
        J.off = 3 * D;  // sin = cos shifted by -D
        J.jlo = 1; J.jhi = N - 1;
        J.klo = 1; J.khi = N - 1;
        if (kind == K_S1_S2F) { J.w0 = J.wm = J.wl = 2.0; J.s0 = J.sm = J.sl = 1.0 / D; }
      }
      break;
    }
    default: {
      const int D = N;
      J.D = D;
      const double inv = 1.0 / N;
      if (kind == K_ZC_S2F) {
        J.aj = 1; J.bj = 0; J.ak = 2; J.bk = 1;
        J.w0 = 1.0; J.wm = 2.0; J.wl = 2.0;
        J.s0 = J.sm = J.sl = inv;
      } else if (kind == K_ZS_S2F) {
        J.aj = 1; J.bj = 1; J.ak = 2; J.bk = 1; J.off = 3 * D;
        J.w0 = 2.0; J.wm = 2.0; J.wl = 1.0;
        J.s0 = J.sm = J.sl = inv;
      } else if (kind == K_ZC_F2S) {
        J.aj = 2; J.bj = 1; J.ak = 1; J.bk = 0;
      } else {  // K_ZS_F2S
        J.aj = 2; J.bj = 1; J.ak = 1; J.bk = 1; J.off = 3 * D;
      }
      break;
    }
  }
}

int axis_kind(int grid_axis_is_z, int dir, int cs) {
  if (grid_axis_is_z) {
    if (dir > 0) return cs ? K_ZS_S2F : K_ZC_S2F;
    return cs ? K_ZS_F2S : K_ZC_F2S;
  }
  if (dir > 0) return cs ? K_S1_S2F : K_C1_S2F;
  return cs ? K_S1_F2S : K_C1_F2S;
}

// FMAs of a two-level pass pair on one line: pass 1 folds k' about A/2,
// pass 2 pairs outputs k, D - k when B is even and every output is wanted
double x_two_level_cost(int A, int B, int D, int nin, int nout) {
  const bool paired = (B % 2 == 0) && nout == D + 1;
  return 2.0 * (A / 2 + 1) * (double)nin + 2.0 * B * (paired ? (double)(D / 2 + 1) : (double)nout);
}
// Choose D = A * B minimising the two-level work x_two_level_cost; A = 0
// when the direct sum (about nin * nout / 2 FMAs) is cheaper.
void pick_factors(int D, int nin, int nout, int* Aout, int* Bout) {
  *Aout = *Bout = 0;
  const double direct = 0.5 * (double)nin * (double)nout;
  double best = 0.6 * direct;  // two passes must pay for the second launch
  for (int A = 2; A <= D / 2; ++A) {
    if (D % A) continue;
    const int B = D / A;
    if (B < 2 || B > 256) continue;  // pass 2 stages B x 32 twiddle pairs
    const double cost = x_two_level_cost(A, B, D, nin, nout);
    if (cost < best) {
      best = cost;
      *Aout = A;
      *Bout = B;
    }
  }
}

// Call f with the smallest batch capacity that holds b's jobs.
template <int NJ>
AxisBatchT<NJ> shrink(const AxisBatch& b) {
  AxisBatchT<NJ> s{};
  for (int i = 0; i < b.njobs; ++i) s.job[i] = b.job[i];
  for (int i = 0; i <= b.njobs; ++i) s.start[i] = b.start[i];
  s.njobs = b.njobs;
  s.early = b.early;
  s.acc = b.acc;
  return s;
}
template <typename F>
void with_capacity(int njobs, F&& f) {
  if (njobs <= 1) f(std::integral_constant<int, 1>{});
  else if (njobs <= 2) f(std::integral_constant<int, 2>{});
  else if (njobs <= 4) f(std::integral_constant<int, 4>{});
  else if (njobs <= 8) f(std::integral_constant<int, 8>{});
  else f(std::integral_constant<int, kMaxJobs>{});
}
template <typename K>
void allow_smem(K kern) {
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// Shared memory of pass 1 for a job with kpc values of k' per cluster and
// ncl CTAs per cluster, and of pass 2 with ncl CTAs per cluster.
size_t pass1_smem(const AxisJob& J, int kpc, int ncl) {
  const int j_end = std::min(J.jhi, J.nin);
  const int K = (j_end + J.B - 1) / J.B;
  const int Kc = p1_slice(K, ncl);
  const int nkp = std::min(kpc, p1_half(J.A) + 1);
  const int items = std::max(kP1Threads, nkp * J.B);
  return sizeof(double) *
         (4 * (size_t)kpc * J.B + (size_t)Kc * J.B + 2 * (size_t)kpc * Kc + 4 * (size_t)items);
}
size_t pass2_smem(const AxisJob& J, int ncl) {
  return sizeof(double) * 2 * 32 * (size_t)p2_slice(J.B, ncl, J.mode == 1);
}

// Cluster size: split a CTA's sum only while its FP64 work (`fmas`, at about
// 2 FMAs per cycle per SM) exceeds the cost of the cluster barriers, the
// launch has room on the SMs, and each CTA keeps at least 4 terms.
int pick_cluster(long long units, long long fmas, int terms, int nsm) {
  int ncl = 1;
  while (ncl < 8 && fmas / ncl > 4096 && units * ncl < 4LL * std::max(nsm, 1) && 2 * ncl * 4 <= terms)
    ncl *= 2;
  return ncl;
}

// FMAs of a two-level pass pair on one line
double two_level_fmas(const AxisJob& J) {
  return x_two_level_cost(J.A, J.B, J.D, std::min(J.nin, J.N), J.nout);
}
// the y passes (ytl_pass1/2) fold and pair the same way (pairing when the
// job's mode is 1)
double y_two_level_fmas(const AxisJob& J) {
  return 2.0 * (J.A / 2 + 1) * (double)std::min(J.nin, J.N) +
         2.0 * J.B * (J.mode == 1 ? (double)(J.D / 2 + 1) : (double)J.nout);
}
// outputs k <= D/2 of one k' class of a y pass are at most this many
bool ytl_can_pair(int D, int A, int B, int nout, int N) {
  return B % 2 == 0 && nout == N && 2 * ((D / 2) / (2 * A)) + 2 <= kYH;
}

void launch_two_level(AxisBatch& b, int nsm, bool early, cudaStream_t st) {
  b.early = early ? 1 : 0;
  for (int i = 0; i < b.njobs; ++i) g_xform_fmas += (double)b.job[i].nlines * two_level_fmas(b.job[i]);
  static PerDeviceOnce attr_set;
  attr_set.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_capacity(nj, [&](auto c) {
        allow_smem(two_level_pass1<decltype(c)::value>);
        allow_smem(two_level_pass2<decltype(c)::value>);
      });
  });
  // pass 1: one k' per cluster while that gives fewer than two clusters per
  // SM, else up to 8 k' per cluster so that each CTA reuses its staged row;
  // the j1 sums are split over a cluster when there are few rows
  long long rows = 0, kbmax = 0;
  int kmin = 1 << 30;
  for (int i = 0; i < b.njobs; ++i) {
    const AxisJob& J = b.job[i];
    rows += (long long)J.nlines * (p1_half(J.A) + 1);
    const int K = (std::min(J.jhi, J.nin) + J.B - 1) / J.B;
    kmin = std::min(kmin, K);
    kbmax = std::max(kbmax, (long long)K * J.B);
  }
  int kpc = (int)std::min<long long>(8, std::max<long long>(1, rows / (2LL * std::max(nsm, 1))));
  const int ncl1 = pick_cluster((rows + kpc - 1) / kpc, 2 * kbmax * kpc, kmin, nsm);
  size_t smem1 = 0, smem2 = 0;
  for (int i = 0; i < b.njobs; ++i) smem1 = std::max(smem1, pass1_smem(b.job[i], kpc, ncl1));
  while (kpc > 1 && smem1 > 160 * 1024) {
    kpc /= 2;
    smem1 = 0;
    for (int i = 0; i < b.njobs; ++i) smem1 = std::max(smem1, pass1_smem(b.job[i], kpc, ncl1));
  }
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    b.start[i] = total;
    total += b.job[i].nlines * ((p1_half(b.job[i].A) + 1 + kpc - 1) / kpc) * ncl1;
  }
  b.start[b.njobs] = total;
  if (total > 0)
    with_capacity(b.njobs, [&](auto c) {
      constexpr int NJ = decltype(c)::value;
      launch_pdl_cluster(two_level_pass1<NJ>, dim3(total), dim3(kP1Threads), smem1, ncl1, st, shrink<NJ>(b),
                         kpc, ncl1);
    });
  // pass 2 with many lines per job: line groups share their staged twiddles
  int minl = 1 << 30;
  for (int i = 0; i < b.njobs; ++i) minl = std::min(minl, b.job[i].nlines);
  if (minl >= 16) {
    static PerDeviceOnce attr_l;
    attr_l.run([&] {
      for (int nj : {1, 2, 4, 8, kMaxJobs})
        with_capacity(nj, [&](auto c) { allow_smem(two_level_pass2_lines<decltype(c)::value>); });
    });
    long long blocks = 0;
    for (int i = 0; i < b.njobs; ++i) blocks += (long long)b.job[i].nlines * ((p2_lanes(b.job[i]) + 31) / 32);
    const int lpc = (int)std::min<long long>(16, std::max<long long>(4, blocks / (4LL * std::max(nsm, 1))));
    total = 0;
    for (int i = 0; i < b.njobs; ++i) {
      b.start[i] = total;
      total += ((b.job[i].nlines + lpc - 1) / lpc) * ((p2_lanes(b.job[i]) + 31) / 32);
      smem2 = std::max(smem2, pass2_smem(b.job[i], 1));
    }
    b.start[b.njobs] = total;
    with_capacity(b.njobs, [&](auto c) {
      constexpr int NJ = decltype(c)::value;
      launch_pdl(two_level_pass2_lines<NJ>, dim3(total), dim3(kP2Threads), smem2, st, shrink<NJ>(b), lpc);
    });
    return;
  }
  // pass 2: 32 outputs per cluster, the j2 sums split over a cluster when
  // there are few output blocks
  long long blocks = 0;
  int bmin = 1 << 30, bmax = 0;
  for (int i = 0; i < b.njobs; ++i) {
    blocks += (long long)b.job[i].nlines * ((p2_lanes(b.job[i]) + 31) / 32);
    bmin = std::min(bmin, b.job[i].B);
    bmax = std::max(bmax, b.job[i].B);
  }
  const int ncl2 = pick_cluster(blocks, 64LL * bmax, bmin, nsm);
  total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    b.start[i] = total;
    total += b.job[i].nlines * ((p2_lanes(b.job[i]) + 31) / 32) * ncl2;
    smem2 = std::max(smem2, pass2_smem(b.job[i], ncl2));
  }
  b.start[b.njobs] = total;
  if (total > 0)
    with_capacity(b.njobs, [&](auto c) {
      constexpr int NJ = decltype(c)::value;
      launch_pdl_cluster(two_level_pass2<NJ>, dim3(total), dim3(kP2Threads), smem2, ncl2, st, shrink<NJ>(b),
                         ncl2);
    });
}

// Shared memory of the fused pass for job J with nsplit CTAs per class pair.
size_t fused_smem(const AxisJob& J, int nsplit) {
  const int j_end = std::min(J.jhi, J.nin);
  const int K = (j_end + J.B - 1) / J.B;
  const int Klp = (K + 1) & ~1;
  const int nlane = J.mode == 1 ? J.D / 2 + 1 : J.nout;
  size_t red = (size_t)4 * fused_p1_parts(J.B) * J.B;
  for (int g = 0; g <= J.A / 2; ++g) {
    const int nslot = fused_slots(J.A, g, nlane);
    const int nu = (nslot + nsplit - 1) / nsplit;
    const int nsb = (nu + 31) / 32;
    red = std::max(red, (size_t)nsb * fused_parts(nsb) * 32);
  }
  return sizeof(double) * (2 * (size_t)J.D + 1 + (size_t)Klp * J.B + 4 * (size_t)J.B + red);
}

// The fused pass serves x-pass batches whose jobs have few lines in all
// (2-D tanks) and no accumulation epilogue, when its shared memory fits;
// returns false (launching nothing) otherwise.
bool launch_two_level_fused(AxisBatch& b, int nsm, bool early, cudaStream_t st) {
  if (!g_fused_enabled) return false;
  long long units = 0;
  for (int i = 0; i < b.njobs; ++i) {
    const AxisJob& J = b.job[i];
    if (J.epi || J.A < 2 || J.wm == 0.0) return false;
    units += (long long)J.nlines * (J.A / 2 + 1);
  }
  if (units == 0 || units > 4LL * std::max(nsm, 1)) return false;
  // a small launch spreads each pair's outputs over up to 4 CTAs
  const int nsplit = (int)std::max<long long>(1, std::min<long long>(4, std::max(nsm, 1) / units));
  size_t smem = 0;
  for (int i = 0; i < b.njobs; ++i) smem = std::max(smem, fused_smem(b.job[i], nsplit));
  if (smem > 200 * 1024) return false;
  static PerDeviceOnce attr_set;
  attr_set.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_capacity(nj, [&](auto c) { allow_smem(two_level_fused<decltype(c)::value>); });
  });
  b.early = early ? 1 : 0;
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    const AxisJob& J = b.job[i];
    b.start[i] = total;
    total += J.nlines * (J.A / 2 + 1) * nsplit;
    // pass 1 runs once per CTA of a pair
    g_xform_fmas += (double)J.nlines * (two_level_fmas(J) +
                                        (nsplit - 1) * 2.0 * (J.A / 2 + 1) * std::min(J.nin, J.N));
  }
  b.start[b.njobs] = total;
  with_capacity(b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    launch_pdl(two_level_fused<NJ>, dim3(total), dim3(kFThreads), smem, st, shrink<NJ>(b), nsplit);
  });
  return true;
}

// Decide the symmetry mode and the split of every x-pass job, then launch.
void launch_batch_x(AxisBatch& b, const Tables& tb, cudaStream_t st) {
  b.early = tb.q_const ? 1 : 0;
  long long tiles_total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    AxisJob& J = b.job[i];
    const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);  // REDFT00 / RODFT00 kinds
    const int D = J.D;
    const int j_end = std::min(J.jhi, J.nin);
    if (c1s1 && J.nout == J.N && D >= 4) {
      J.mode = 1;
      J.nlane = D / 2 + 1;
      J.ta = std::max(J.jlo, 1);
      J.tb = std::min(j_end, J.N - 1);
    } else if (c1s1 && J.nin >= J.N && J.nout <= D / 2 + 1 && D >= 4 &&
               J.w0 == J.wl) {
      J.mode = 2;
      J.nlane = J.nout;
      J.ta = std::max(J.jlo, 1);
      J.tb = (D + 1) / 2;  // pairs j < D - j
    } else {
      J.mode = 0;
      J.nlane = J.nout;
      J.ta = std::max(J.jlo, 1);
      J.tb = std::min(j_end, J.N - 1);
    }
    if (J.tb < J.ta) J.tb = J.ta;
    J.ntile = (J.nlane + 31) / 32;
    tiles_total += (long long)J.nlines * J.ntile;
  }
  const long long target = 4LL * std::max(tb.nsm, 1);
  long long part_need = 0, cnt_need = 0;
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    AxisJob& J = b.job[i];
    int terms = J.tb - J.ta;
    int nchunk = 1;
    if (tiles_total < target && terms > 512)
      nchunk = std::min((int)((target + tiles_total - 1) / tiles_total), (terms + 255) / 256);
    int chunk = std::max(1, (terms + nchunk - 1) / std::max(nchunk, 1));
    nchunk = std::max(1, (terms + chunk - 1) / chunk);
    J.part = nullptr;
    J.cnt = nullptr;
    if (nchunk > 1) {
      const long long np = (long long)J.nlines * J.ntile * nchunk * 64;
      const long long nc = (long long)J.nlines * J.ntile;
      if (part_need + np <= tb.part_cap && cnt_need + nc <= tb.cnt_cap) {
        J.part = tb.part + part_need;
        J.cnt = tb.cnt + cnt_need;
        part_need += np;
        cnt_need += nc;
      } else {
        // not enough scratch for a split sum: one CTA per tile
        nchunk = 1;
        chunk = std::max(terms, 1);
      }
    }
    J.nchunk = nchunk;
    J.chunk = chunk;
    g_xform_fmas += (double)J.nlines * J.nlane * std::max(J.tb - J.ta, 1);
    b.start[i] = total;
    total += J.nlines * J.ntile * J.nchunk;
  }
  b.start[b.njobs] = total;
  size_t smem = 0;
  for (int i = 0; i < b.njobs; ++i)
    smem = std::max(smem, sizeof(double) * ((size_t)b.job[i].D + 1 + 2 * (size_t)kMaxPairChunk));
  static PerDeviceOnce attr_set;
  attr_set.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_capacity(nj, [&](auto c) { allow_smem(axis_pass_lanes_k<decltype(c)::value>); });
  });
  if (total > 0)
    with_capacity(b.njobs, [&](auto c) {
      constexpr int NJ = decltype(c)::value;
      launch_pdl(axis_pass_lanes_k<NJ>, dim3(total), dim3(kXThreads), smem, st, shrink<NJ>(b));
    });
}

// Factor pair of a y pass: minimum 2 (A+1) nin + 2 B nout FMAs, with every
// k' class (at most 2 nout / (2A) + 2 outputs) held by one pass-2 thread;
// A = 0 when the direct sum (nin * nout FMAs) is cheaper.
void pick_factors_y(int D, int nin, int nout, int* Aout, int* Bout) {
  *Aout = *Bout = 0;
  double best = 0.6 * (double)nin * (double)nout;
  for (int A = 2; A <= D / 2; ++A) {
    if (D % A) continue;
    const int B = D / A;
    if (B < 2 || B > 256) continue;
    if (2 * ((nout + 2 * A - 1) / (2 * A)) + 1 > kYQ) continue;
    const bool paired = ytl_can_pair(D, A, B, nout, D + 1);
    const double cost = 2.0 * (A / 2 + 1) * (double)nin + 2.0 * B * (paired ? (double)(D / 2 + 1) : (double)nout);
    if (cost < best) {
      best = cost;
      *Aout = A;
      *Bout = B;
    }
  }
}

void launch_ytl(AxisBatch& b, bool early, cudaStream_t st) {
  b.early = early ? 1 : 0;
  for (int i = 0; i < b.njobs; ++i) g_xform_fmas += (double)b.job[i].nlines * y_two_level_fmas(b.job[i]);
  static PerDeviceOnce attr_set;
  attr_set.run([&] {
    for (int nj : {1, 2, 4, 8, kMaxJobs})
      with_capacity(nj, [&](auto c) {
        allow_smem(ytl_pass1<decltype(c)::value>);
        allow_smem(ytl_pass2<decltype(c)::value>);
      });
  });
  int total = 0;
  size_t smem1 = 0, smem2 = 0;
  for (int i = 0; i < b.njobs; ++i) {
    const AxisJob& J = b.job[i];
    const int nlb = (J.nlines + kYT - 1) / kYT;
    const int K = (std::min(J.jhi, J.nin) + J.B - 1) / J.B;
    b.start[i] = total;
    total += nlb * J.B * ((J.A / 2 + 1 + kYKF - 1) / kYKF);
    smem1 = std::max(smem1, sizeof(double) * 2 * (size_t)((K + 1) & ~1) * kYKF);
    smem2 = std::max(smem2, sizeof(double) * 2 * (size_t)J.B * kYQ);
  }
  b.start[b.njobs] = total;
  with_capacity(b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    launch_pdl(ytl_pass1<NJ>, dim3(total), dim3(kYT), smem1, st, shrink<NJ>(b));
  });
  total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    b.start[i] = total;
    total += ((b.job[i].nlines + kYT - 1) / kYT) * (b.job[i].A + 1);
  }
  b.start[b.njobs] = total;
  with_capacity(b.njobs, [&](auto c) {
    constexpr int NJ = decltype(c)::value;
    launch_pdl(ytl_pass2<NJ>, dim3(total), dim3(kYT), smem2, st, shrink<NJ>(b));
  });
}

// y passes: two-level where the length factors well (scratch permitting),
// direct sums otherwise
void launch_batch_y(AxisBatch& in, const Tables& tb, cudaStream_t st) {
  AxisBatch b{}, b2{}, bf{};
  b.njobs = b2.njobs = bf.njobs = 0;
  b.acc = b2.acc = bf.acc = in.acc;
  const FftPlanInfo* fplan[kMaxJobs];
  long long cs_used = 0;
  for (int i = 0; i < in.njobs; ++i) {
    AxisJob J = in.job[i];
    J.A = J.B = 0;
    J.cs = nullptr;
    const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);
    if (c1s1) {
      const int nin = std::min(J.nin, J.N);
      int A = 0, B = 0;
      pick_factors_y(J.D, nin, J.nout, &A, &B);
      double other = 0.5 * (double)nin * J.nout;
      if (A > 0) {
        J.A = A;
        J.B = B;
        J.mode = ytl_can_pair(J.D, A, B, J.nout, J.N) ? 1 : 0;
        other = y_two_level_fmas(J);
        J.A = J.B = 0;
        J.mode = 0;
      }
      if (const FftPlanInfo* f = fft_choice(J, tb, other)) {
        fplan[bf.njobs] = f;
        bf.job[bf.njobs++] = J;
        continue;
      }
    }
    if (c1s1 && tb.cs) {
      int A = 0, B = 0;
      pick_factors_y(J.D, std::min(J.nin, J.N), J.nout, &A, &B);
      const long long need = (long long)J.nlines * B * (A + 1) * 2;
      if (A > 0 && cs_used + need <= tb.cs_cap) {
        J.A = A;
        J.B = B;
        J.mode = ytl_can_pair(J.D, A, B, J.nout, J.N) ? 1 : 0;
        J.cs = tb.cs + cs_used;
        cs_used += need;
        b2.job[b2.njobs++] = J;
        continue;
      }
    }
    b.job[b.njobs++] = J;
  }
  if (bf.njobs) launch_fft_jobs(bf, fplan, tb, st);
  if (b2.njobs) launch_ytl(b2, tb.q_const, st);
  if (b.njobs == 0) return;
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    AxisJob& J = b.job[i];
    const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);
    J.mode = 0;
    J.nlane = J.nout;
    if (c1s1 && J.nout == J.N && J.D >= 4) {
      J.mode = 1;
      J.nlane = J.D / 2 + 1;
    } else if (c1s1 && J.nin >= J.N && J.nout <= J.D / 2 + 1 && J.D >= 4 && J.w0 == J.wl) {
      J.mode = 2;
    }
    {
      const int nin = std::min(std::min(J.jhi, J.nin), J.N) - J.jlo;
      g_xform_fmas += (double)J.nlines * J.nlane * (J.mode == 2 ? (J.D + 1) / 2 : std::max(nin, 1));
    }
    b.start[i] = total;
    const int nlb = (J.nlines + kYThreads - 1) / kYThreads;
    total += nlb * ((J.nlane + kYR - 1) / kYR);
  }
  b.start[b.njobs] = total;
  if (total > 0)
    with_capacity(b.njobs, [&](auto c) {
      constexpr int NJ = decltype(c)::value;
      launch_pdl(axis_pass_lanes_line<NJ>, dim3(total), dim3(kYThreads), 0, st, shrink<NJ>(b));
    });
}

}  // namespace

thread_local double g_xform_fmas = 0.0;
thread_local bool g_launch_no_pdl = false;
const bool g_fused_enabled = [] {
  const char* e = std::getenv("HOSNWT_FUSED_PASS");
  return e && e[0] == '1';
}();

std::vector<double> quarter_table(int D) {
  std::vector<double> q(D + 1);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int m = 0; m <= D; ++m) {
    q[m] = (double)cosl(pi * (long double)m / (2.0L * (long double)D));
  }
  if (D > 0) q[D] = 0.0;
  if (D % 3 == 0) q[2 * D / 3] = 0.5;  // cos(pi/3)
  return q;
}

std::vector<double> y_twiddle_rows(int N, bool sin_kind, int* ld) {
  const int D = N - 1;
  const int nk = D / 2 + 1;
  *ld = (nk + 7) / 8 * 8;
  const std::vector<double> q = quarter_table(D);
  std::vector<double> t((size_t)N * *ld, 0.0);
  const long long D4 = 4LL * D, off = sin_kind ? 3LL * D : 0;
  for (int j = 0; j < N; ++j)
    for (int k = 0; k < nk; ++k) {
      const long long m = (2LL * j * k + off) % D4;
      const long long mm = (m > 2LL * D) ? D4 - m : m;
      t[(size_t)j * *ld + k] = (mm > D) ? -q[2 * D - mm] : q[mm];
    }
  return t;
}

namespace {

// The passes of the requests idx[0..n), along x then y.  The first pass
// applies the input weights, the last the scale and the accumulation
// epilogue; tmp[idx[i]] holds the intermediate.
void launch_ordered(const XfReq* reqs, const int* idx, int n, const Tables& tb, double* const* tmp,
                    cudaStream_t st) {
  AxisBatch bx{}, by{};
  bx.njobs = by.njobs = 0;
  for (int i = 0; i < n; ++i)
    if (reqs[idx[i]].acc) bx.acc = by.acc = *reqs[idx[i]].acc;
  for (int i = 0; i < n; ++i) {
    const int r = idx[i];
    const XfReq& R = reqs[r];
    int Nx, Ny;
    const double *qx, *qy;
    const bool zaxis = (R.grid == GRID_ADD);
    if (R.grid == GRID_N) { Nx = tb.n1; Ny = tb.n2; qx = tb.q_n1; qy = tb.q_n2; }
    else if (R.grid == GRID_BIG) { Nx = tb.nd1; Ny = tb.nd2; qx = tb.q_nd1; qy = tb.q_nd2; }
    else { Nx = tb.n3_add; Ny = tb.n2; qx = tb.q_add; qy = tb.q_n2; }
    const bool twod = (tb.n2 != 1);
    // x (or z) pass
    AxisJob& X = bx.job[bx.njobs++];
    set_kind(X, axis_kind(zaxis, R.dir, R.csx), Nx, qx);
    X.nin = R.nin1;
    X.nout = R.nout1;
    X.out_sk = 1;
    X.win_sk = 1;
    if (!twod) {
      X.in = R.in;
      X.in_sk = 1;
      X.in_sl = R.in_ld;
      X.win = R.win;
      X.win_sl = R.win_ld;
      X.nlines = 1;
      X.out = R.out;
      X.out_sl = R.out_ld;
      X.gscale = R.scale;
      X.epi = R.acc ? 1 : 0;
      continue;
    }
    AxisJob& Y = by.job[by.njobs++];
    set_kind(Y, axis_kind(false, R.dir, R.csy), Ny, qy);
    Y.ty = (R.grid == GRID_BIG) ? tb.ty_nd2[R.csy ? 1 : 0] : tb.ty_n2[R.csy ? 1 : 0];
    Y.ldy = (R.grid == GRID_BIG) ? tb.ldy_nd2 : tb.ldy_n2;
    Y.nin = R.nin2;
    Y.nout = R.nout2;
    Y.out_sl = 1;
    // The y-sin plans zero the boundary columns of the input and output
    // (fourier_FFTW.f90:282-285, 296-299): the x pass skips the lines beyond
    // the input's extent.
    X.in = R.in;
    X.in_sk = 1;
    X.in_sl = R.in_ld;
    X.win = R.win;
    X.win_sl = R.win_ld;
    X.nlines = R.nin2;
    X.out = tmp[r];
    X.out_sl = R.nout1;
    X.gscale = 1.0;
    X.epi = 0;
    Y.in = tmp[r];
    Y.in_sk = R.nout1;
    Y.in_sl = 1;
    Y.nlines = R.nout1;
    Y.out = R.out;
    Y.out_sk = R.out_ld;
    Y.gscale = R.scale;
    Y.epi = R.acc ? 1 : 0;
  }
  // FFT passes for the x jobs over many lines where they cost less, then
  // two-level passes for the jobs whose length factors well
  AxisBatch b2{}, bd{}, bf{};
  b2.njobs = bd.njobs = bf.njobs = 0;
  b2.acc = bd.acc = bf.acc = bx.acc;
  const FftPlanInfo* fplan[kMaxJobs];
  long long cs_used = 0;
  for (int i = 0; i < bx.njobs; ++i) {
    AxisJob J = bx.job[i];
    J.A = J.B = 0;
    J.cs = nullptr;
    const bool c1s1 = (J.aj == 2 && J.bj == 0 && J.ak == 1 && J.bk == 0);
    if (c1s1) {
      const int nin = std::min(J.nin, J.N);
      int A = 0, B = 0;
      pick_factors(J.D, nin, J.nout, &A, &B);
      const double other = A > 0 ? x_two_level_cost(A, B, J.D, nin, J.nout) : 0.5 * (double)nin * J.nout;
      if (const FftPlanInfo* f = fft_choice(J, tb, other)) {
        fplan[bf.njobs] = f;
        bf.job[bf.njobs++] = J;
        continue;
      }
    }
    if (c1s1 && tb.cs) {
      int A = 0, B = 0;
      pick_factors(J.D, std::min(J.nin, J.N), J.nout, &A, &B);
      const long long need = (long long)J.nlines * B * (A + 1) * 2;
      if (A > 0 && cs_used + need <= tb.cs_cap) {
        J.A = A;
        J.B = B;
        J.mode = (B % 2 == 0 && J.nout == J.N) ? 1 : 0;  // pass 2 pairs k, D - k
        J.cs = tb.cs + cs_used;
        cs_used += need;
        b2.job[b2.njobs++] = J;
        continue;
      }
    }
    bd.job[bd.njobs++] = J;
  }
  if (bf.njobs) launch_fft_jobs(bf, fplan, tb, st);
  if (b2.njobs && !launch_two_level_fused(b2, tb.nsm, tb.q_const, st))
    launch_two_level(b2, tb.nsm, tb.q_const, st);
  if (bd.njobs) launch_batch_x(bd, tb, st);
  if (by.njobs) launch_batch_y(by, tb, st);
}

}  // namespace

void launch_transforms(const XfReq* reqs, int nreq, const Tables& tb, double* const* tmp,
                       cudaStream_t st) {
  // x then y for every request.  (Running the y pass first, where it takes
  // fewer FMAs, was measured slower on the 3-D big grid: the x pass over
  // the extra lines runs at a lower FP64 rate than the y pass it saves.)
  int idx[kMaxJobs];
  for (int r = 0; r < nreq; ++r) idx[r] = r;
  launch_ordered(reqs, idx, nreq, tb, tmp, st);
}

namespace {
__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  pdl_wait();
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

double measure_fp64_peak_gflops() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4, threads = 256, iters = 2048;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_dfma_peak<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  return flops / (best * 1e-3) / 1e9;
}

void launch_y_f2s(const Tables& tb, const double* in, int nlines, long long y_stride, double* out,
                  long long out_y_stride, int cs, cudaStream_t st) {
  AxisBatch b{};
  b.njobs = 1;
  AxisJob& J = b.job[0];
  set_kind(J, cs ? K_S1_F2S : K_C1_F2S, tb.n2, tb.q_n2);
  J.ty = tb.ty_n2[cs ? 1 : 0];
  J.ldy = tb.ldy_n2;
  J.in = in;
  J.in_sk = y_stride;
  J.in_sl = 1;
  J.nin = tb.n2;
  J.nlines = nlines;
  J.nout = tb.n2;
  J.out = out;
  J.out_sk = out_y_stride;
  J.out_sl = 1;
  J.gscale = 1.0;
  launch_batch_y(b, tb, st);
}

}  // namespace hos
