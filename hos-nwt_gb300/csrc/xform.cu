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
#include <cmath>

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

constexpr int kXThreads = 256;   // 8 warps
constexpr int kXWarps = kXThreads / 32;

// x pass: one CTA = (job, line, tile of 32 outputs); the 8 warps split the
// summation range, lanes own outputs.
__global__ void __launch_bounds__(kXThreads) axis_pass_lanes_k(const AxisBatch b) {
  __shared__ double red[kXWarps][32];
  int jb = 0;
  while (jb + 1 < b.njobs && (int)blockIdx.x >= b.start[jb + 1]) ++jb;
  const AxisJob& J = b.job[jb];
  const int local = blockIdx.x - b.start[jb];
  const int ntile = (J.nout + 31) / 32;
  const int line = local / ntile;
  const int tile = local - line * ntile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = tile * 32 + lane;
  const int D4 = 4 * J.D;
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;

  double acc = 0.0;
  const bool active = (k < J.nout) && (k >= J.klo) && (k < J.khi);
  if (active) {
    const int j_end = min(J.jhi, J.nin);
    const int kk = J.ak * k + J.bk;
    // interior range [max(jlo,1), min(j_end, N-1)) split over warps
    const int a0 = max(J.jlo, 1), a1 = min(j_end, J.N - 1);
    if (a1 > a0) {
      const int len = a1 - a0;
      const int chunk = (len + kXWarps - 1) / kXWarps;
      const int ja = a0 + warp * chunk;
      const int jz = min(a1, ja + chunk);
      if (jz > ja) {
        int m = mod4d((long long)(J.aj * ja + J.bj) * kk + J.off, D4);
        const int inc = mod4d((long long)J.aj * kk, D4);
        double s = 0.0;
        const double* __restrict__ xp = x + (long long)ja * J.in_sk;
        for (int j = ja; j < jz; ++j) {
          s = fma(__ldg(xp), twiddle(J.q, J.D, m), s);
          xp += J.in_sk;
          m += inc;
          if (m >= D4) m -= D4;
        }
        acc = J.wm * s;
      }
    }
    if (warp == 0) {
      if (J.jlo == 0 && 0 < j_end) {
        const int m = mod4d((long long)J.bj * kk + J.off, D4);
        acc = fma(J.w0 * __ldg(x), twiddle(J.q, J.D, m), acc);
      }
      const int jl = J.N - 1;
      if (jl > 0 && jl >= J.jlo && jl < j_end) {
        const int m = mod4d((long long)(J.aj * jl + J.bj) * kk + J.off, D4);
        acc = fma(J.wl * __ldg(x + (long long)jl * J.in_sk), twiddle(J.q, J.D, m), acc);
      }
    }
  }
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && k < J.nout) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kXWarps; ++w) t += red[w][lane];
    double sc = (k == 0) ? J.s0 : ((k == J.N - 1) ? J.sl : J.sm);
    double v = active ? t * sc * J.gscale : 0.0;
    J.out[(long long)line * J.out_sl + (long long)k * J.out_sk] = v;
  }
}

constexpr int kYThreads = 128;
constexpr int kYR = 8;  // outputs per thread

// y pass: one thread = one line (consecutive lines are contiguous in memory)
// and kYR outputs; twiddles are warp-uniform.
__global__ void __launch_bounds__(kYThreads) axis_pass_lanes_line(const AxisBatch b) {
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
  const int D4 = 4 * J.D;
  const double* __restrict__ x = J.in + (long long)line * J.in_sl;
  const int j_end = min(J.jhi, J.nin);

  double acc[kYR];
  int m[kYR], inc[kYR];
#pragma unroll
  for (int r = 0; r < kYR; ++r) {
    acc[r] = 0.0;
    const int kk = J.ak * (k0 + r) + J.bk;
    inc[r] = mod4d((long long)J.aj * kk, D4);
    const int ja = max(J.jlo, 1);
    m[r] = mod4d((long long)(J.aj * ja + J.bj) * kk + J.off, D4);
  }
  const int a0 = max(J.jlo, 1), a1 = min(j_end, J.N - 1);
  for (int j = a0; j < a1; ++j) {
    const double v = __ldg(x + (long long)j * J.in_sk);
#pragma unroll
    for (int r = 0; r < kYR; ++r) {
      acc[r] = fma(v, twiddle(J.q, J.D, m[r]), acc[r]);
      m[r] += inc[r];
      if (m[r] >= D4) m[r] -= D4;
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
      t = fma(J.w0 * __ldg(x), twiddle(J.q, J.D, mm), t);
    }
    const int jl = J.N - 1;
    if (jl > 0 && jl >= J.jlo && jl < j_end) {
      const int mm = mod4d((long long)(J.aj * jl + J.bj) * kk + J.off, D4);
      t = fma(J.wl * __ldg(x + (long long)jl * J.in_sk), twiddle(J.q, J.D, mm), t);
    }
    const bool active = (k >= J.klo) && (k < J.khi);
    const double sc = (k == 0) ? J.s0 : ((k == J.N - 1) ? J.sl : J.sm);
    J.out[(long long)line * J.out_sl + (long long)k * J.out_sk] = active ? t * sc * J.gscale : 0.0;
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

void launch_batch_x(AxisBatch& b, cudaStream_t st) {
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    b.start[i] = total;
    total += b.job[i].nlines * ((b.job[i].nout + 31) / 32);
  }
  b.start[b.njobs] = total;
  if (total > 0) axis_pass_lanes_k<<<total, kXThreads, 0, st>>>(b);
}

void launch_batch_y(AxisBatch& b, cudaStream_t st) {
  int total = 0;
  for (int i = 0; i < b.njobs; ++i) {
    b.start[i] = total;
    const int nlb = (b.job[i].nlines + kYThreads - 1) / kYThreads;
    total += nlb * ((b.job[i].nout + kYR - 1) / kYR);
  }
  b.start[b.njobs] = total;
  if (total > 0) axis_pass_lanes_line<<<total, kYThreads, 0, st>>>(b);
}

}  // namespace

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

void launch_transforms(const XfReq* reqs, int nreq, const Tables& tb, double* const* tmp,
                       cudaStream_t st) {
  AxisBatch bx{}, by{};
  bx.njobs = by.njobs = 0;
  for (int r = 0; r < nreq; ++r) {
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
    X.in = R.in;
    X.in_sk = 1;
    X.in_sl = R.in_ld;
    X.nin = R.nin1;
    X.gscale = twod ? 1.0 : R.scale;
    if (twod) {
      // the y-sin plans zero the boundary columns of the input and output
      // (fourier_FFTW.f90:282-285, 296-299): skip those lines here
      X.nlines = R.nin2;
      X.nout = R.nout1;
      X.out = tmp[r];
      X.out_sk = 1;
      X.out_sl = R.nout1;
    } else {
      X.nlines = 1;
      X.nout = R.nout1;
      X.out = R.out;
      X.out_sk = 1;
      X.out_sl = R.out_ld;
    }
    if (twod) {
      AxisJob& Y = by.job[by.njobs++];
      set_kind(Y, axis_kind(false, R.dir, R.csy), Ny, qy);
      Y.in = tmp[r];
      Y.in_sk = R.nout1;
      Y.in_sl = 1;
      Y.nin = R.nin2;
      Y.nlines = R.nout1;
      Y.nout = R.nout2;
      Y.out = R.out;
      Y.out_sk = R.out_ld;
      Y.out_sl = 1;
      Y.gscale = R.scale;
    }
  }
  launch_batch_x(bx, st);
  if (by.njobs) launch_batch_y(by, st);
}

void launch_y_f2s(const Tables& tb, const double* in, int nlines, long long y_stride, double* out,
                  long long out_y_stride, int cs, cudaStream_t st) {
  AxisBatch b{};
  b.njobs = 1;
  AxisJob& J = b.job[0];
  set_kind(J, cs ? K_S1_F2S : K_C1_F2S, tb.n2, tb.q_n2);
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
  launch_batch_y(b, st);
}

}  // namespace hos
