// Nonlinear right-hand side, wavemaker potential and RK4(5) step of the HOS
// wave tank on sm_103a (FP64 throughout).
//
//   solveHOS2        resol_HOS.f90:270-656      enqueue_rhs
//   phisxy_etaxy     resol_HOS.f90:924-1078     (batch A transforms + powers)
//   HOSphis_modes    resol_HOS.f90:665-915      (order loop)
//   dealias/filter   dealiasing.f90:39-134      dealias(), filters
//   SWEET_1          resol_wmkr.f90:109-210     wavemaker block
//   phiadd_SL        resol_wmkr.f90:1124-1187   k_phiadd_*
//   ramp / pos_1st   resol_wmkr.f90:1268-1397, wavemaking.f90:259-304
//   runge4_adapt2    runge_kutta.f90:81-360     enqueue_step
//   GtoF / expon     variablechange.f90:37-130
//
// Linear combinations that the reference filters separately are filtered
// once (filter_ext is linear), and the S2F that follows a dealiasing is
// fused with its truncation; both only change rounding.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include "tank.h"

namespace hos {

namespace {

constexpr int kEW = 256;
// FP64 sincos per element is slow on this part: kernels that evaluate one per
// element use small blocks so that the work spreads over more SMs.
constexpr int kTrig = 64;
inline int nblk(long long n, int t = kEW) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// deterministic "last block" reductions (no spin-waits)
// ---------------------------------------------------------------------------
// Maximum that keeps a NaN (fmax drops it): a NaN anywhere in a reduced
// field reaches the error estimate, which the step control rejects as
// non-finite (HOSNWT_ERR_NAN).
__device__ __forceinline__ double nan_max(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }

template <int OP>  // 0 sum, 1 max
__device__ double block_reduce(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_down_sync(0xffffffffu, v, o);
    v = OP == 0 ? v + u : nan_max(v, u);
  }
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
    v = lane < nw ? sh[lane] : (OP == 0 ? 0.0 : 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_down_sync(0xffffffffu, v, o);
      v = OP == 0 ? v + u : nan_max(v, u);
    }
  }
  return v;  // valid in thread 0
}

// returns true in thread 0 of the last block to finish
__device__ bool last_block(unsigned int* counter) {
  __shared__ bool amlast;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(counter, 1u);
    amlast = (t == gridDim.x - 1);
  }
  __syncthreads();
  return amlast;
}

__device__ void volume_fix(double* etam, double S, const double* sc, int igeom, double d_hinge,
                           double xlen) {
  const double alpha = sc[SC_ALPHA], pt = sc[SC_POSTOP];
  double v;
  if (igeom == 2)
    v = 0.5 * alpha * (1 - d_hinge) * pt / xlen + S * alpha * pt / xlen;
  else if (igeom == 1)
    v = alpha * pt / xlen + S * alpha * pt / xlen;
  else
    v = 0.0;
  etam[0] = v;
}

// GtoF at the stage start, phis/omega, the volume correction of eta's mean
// mode (resol_HOS.f90:337-364) and the weighted modes -kx*eta, -ky*eta,
// -kx*phis, -ky*phis that feed the big-grid derivatives.
__global__ void k_gtof(const double* __restrict__ G1, const double* __restrict__ G2,
                       const double* __restrict__ om, const double* __restrict__ kx,
                       const double* __restrict__ ky, double* sc_, int n1, int n2, int igeom,
                       double d_hinge, double xlen, double* etam, double* phim, double* wex,
                       double* wey, double* wpx, double* wpy, double* part, unsigned int* counter) {
  pdl_wait();
  const double* sc = sc_;
  const double dt = sc[SC_DT];
  const long long n = (long long)n1 * n2;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < n) {
    const double w = om[i];
    double s, c;
    sincos(-w * dt, &s, &c);
    const double g1 = G1[i], g2 = G2[i];
    e = g1 * c - g2 * s;
    double p = g2 * c + g1 * s;
    if (i != 0) p = p / w;
    etam[i] = e;
    phim[i] = p;
    const int i1 = (int)(i % n1), i2 = (int)(i / n1);
    wex[i] = -kx[i1] * e;
    wey[i] = -ky[i2] * e;
    wpx[i] = -kx[i1] * p;
    wpy[i] = -ky[i2] * p;
  }
  const double bs = block_reduce<0>(e);
  if (threadIdx.x == 0) part[blockIdx.x] = bs;
  if (last_block(counter) && threadIdx.x == 0) {
    double S = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) S += __ldcg(part + b);
    volume_fix(etam, S, sc, igeom, d_hinge, xlen);
    *counter = 0;
  }
}

// eta^j / j! for a run of orders without dealiasing in between:
// e_{j+1} = e_j / (j+1) * e_1 for j = j0 .. j1-1 (resol_HOS.f90:979-987)
struct PowArgs {
  double* e[16];
  int j0, j1;
};
__global__ void k_pow_run(PowArgs a, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double e1 = a.e[0][i];
  double v = a.e[a.j0 - 1][i];
  for (int j = a.j0; j < a.j1; ++j) {
    v = v / (double)(j + 1) * e1;
    a.e[j][i] = v;
  }
}

// Products of HOSphis_modes' quadratic terms accumulated per dealiasing
// group: out[g] = sum over the group's terms of s * x * y (x, y big-grid
// fields); the terms of each group keep the reference's order.
// Optionally also the outer sums oscale * (sum of the groups q with
// outer_of[q] == u), u < nouter: the geta2phiz2 sums of groups that are
// not dealiased themselves, in the order of k_sum_fields.
struct GroupTerms {
  const double* x[48];
  const double* y[48];
  double s[48];
  int group[48];
  int nterm;
  double* out[16];
  int ngroup;
  int outer_of[16];
  double* out_outer[4];
  const double* oscale;
  int nouter;
};
__global__ void k_group_products(GroupTerms g, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.0;
  for (int t = 0; t < g.nterm; ++t) {
    const double v = (g.s[t] * g.x[t][i]) * g.y[t][i];
#pragma unroll
    for (int q = 0; q < 16; ++q)
      if (q == g.group[t]) acc[q] += v;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q)
    if (q < g.ngroup) g.out[q][i] = acc[q];
  if (g.nouter > 0) {
    double os[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      if (q >= g.ngroup) break;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u == g.outer_of[q]) os[u] += acc[q];
    }
    const double sc = g.oscale[i];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (u < g.nouter) g.out_outer[u][i] = sc * os[u];
  }
}

// out = sum of listed fields, optionally times gradeta2 (scale field)
struct SumArgs {
  const double* in[16];
  int nin;
  const double* scale;
  double* out;
};
__global__ void k_sum_fields(SumArgs a, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = 0.0;
  for (int t = 0; t < a.nin; ++t) v += a.in[t][i];
  if (a.scale) v = a.scale[i] * v;
  a.out[i] = v;
}

// out = s * x * y  (s applied first, as 2.0_rp * a * b in the reference)
__global__ void k_mul(const double* __restrict__ x, const double* __restrict__ y, double s,
                      double* out, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (s * x[i]) * y[i];
}

__global__ void k_sq2(const double* __restrict__ a, const double* __restrict__ b, double* out,
                      long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] * a[i] + b[i] * b[i];
}

// products a(m) * kth_ext(:,:,j) on the nonzero extent of a(m)
// order iHOS of HOSphis_modes (resol_HOS.f90:716-764)
struct AccArgs {
  const double* phizi[16];  // phizi(m = iHOS+1-j, j), indexed by j-1
  const double* etapm[16];  // eta^j/j!, indexed by j-1
  int iHOS;
};
__global__ void k_hos_accum(AccArgs a, double* phimext, double* phizm, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double pm = 0.0, pz = 0.0;
  for (int j = a.iHOS; j >= 2; --j) {
    const double z = a.phizi[j - 1][i];
    pm = pm - z * a.etapm[j - 1][i];
    pz = pz + z * a.etapm[j - 2][i];
  }
  const double z1 = a.phizi[0][i];
  phimext[i] = pm - z1 * a.etapm[0][i];
  phizm[i] = pz + z1;
}

__global__ void k_fs_products(const double* __restrict__ etax, const double* __restrict__ etay,
                              const double* __restrict__ phisx, const double* __restrict__ phisy,
                              double* detext, double* dphext, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double px = phisx[i], py = phisy[i];
  detext[i] = -px * etax[i] - py * etay[i];
  dphext[i] = -px * px - py * py;
}

// A1 = detext + geta2phiz + phizMm1 + phizm(M) - grad eta.grad phi_add
// A3 = 0.5 * (dphext + geta2phiz2 + phiz2) - grad phis.grad phi_add - |grad phi_add|^2/2
// (resol_HOS.f90:382-399, 534-608 before filter_ext, which is linear).
// detext / dphext are the order-2 products -grad phis.grad eta, -|grad phis|^2,
// computed here unless the caller dealiased them (p = 2).
struct AssembleArgs {
  const double *etax, *etay, *phisx, *phisy, *pxe, *pye, *pze;
  const double *detext, *dphext;
  const double* phizm[16];  // phizm(1 .. M-1), summed to phizMm1
  int nphizm;
  const double* phizmM;
  const double* g1[8];      // parts of geta2phiz
  int ng1;
  const double* g2[8];      // parts of geta2phiz2
  int ng2;
  const double* t1[16];     // parts of phiz2
  int nt1;
  int M;
};
__global__ void k_assemble(AssembleArgs a, double* A1, double* A3, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ex = a.etax[i], ey = a.etay[i], px = a.phisx[i], py = a.phisy[i];
  const double ax = a.pxe[i], ay = a.pye[i], az = a.pze[i];
  const double gg = ex * ax + ey * ay;
  const double gpg = px * ax + py * ay + 0.5 * (ax * ax + ay * ay + az * az);
  double det = a.detext ? a.detext[i] : (-px * ex - py * ey);
  double dph = a.dphext ? a.dphext[i] : (-px * px - py * py);
  for (int t = 0; t < a.ng1; ++t) det += a.g1[t][i];
  for (int t = 0; t < a.ng2; ++t) dph += a.g2[t][i];
  for (int t = 0; t < a.nt1; ++t) dph += a.t1[t][i];
  if (a.M >= 2) {
    double mm1 = 0.0;
    for (int t = 0; t < a.nphizm; ++t) mm1 += a.phizm[t][i];
    A1[i] = det + mm1 + a.phizmM[i] - gg;
    A3[i] = 0.5 * dph - gpg;
  } else {
    A1[i] = a.phizmM[i];
    A3[i] = 0.0;
  }
}

// final free-surface RHS in physical space (resol_HOS.f90:557-608)
__global__ void k_final(const double* __restrict__ X1, const double* __restrict__ X2,
                        const double* __restrict__ X3, const double* __restrict__ phiz_add,
                        const double* __restrict__ phit_add, const double* __restrict__ nu,
                        double* det, double* dph, long long n, int M) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dphin = X1[i] + phiz_add[i];
  det[i] = dphin - X2[i];
  if (M >= 2)
    dph[i] = X3[i] - phit_add[i] - nu[i] * dphin;
  else
    dph[i] = -phit_add[i] - nu[i] * dphin;
}

// expon (variablechange.f90:37-80) with dG2(1,1) from the unscaled NL2
__global__ void k_expon(const double* __restrict__ NL1, const double* __restrict__ NL2,
                        const double* __restrict__ om, const double* __restrict__ sc, double* kG1,
                        double* kG2, long long n, int rk_mode) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dt = sc[SC_DT];
  const double w = om[i];
  double s, c;
  sincos(w * dt, &s, &c);
  const double a = NL1[i], b0 = NL2[i];
  const double b = b0 * w;
  kG1[i] = a * c - b * s;
  double g2 = b * c + a * s;
  if (i == 0) g2 = rk_mode ? 0.0 : b0;
  kG2[i] = g2;
}

// ---------------------------------------------------------------------------
// wavemaker
// ---------------------------------------------------------------------------
struct RampP {
  int iramp;
  double Tramp, T_stop, T_mono;
};

// ramp (resol_wmkr.f90:1268-1397)
__device__ void ramp_law(const RampP& r, double time, double* a, double* at, double* att) {
  const double Tramp = r.Tramp;
  if (r.iramp == 11) {
    const double T_swtt = 3.0 / sqrt(5.0 / 9.81);
    if (time <= T_swtt) { *a = time / T_swtt; *at = 1.0 / T_swtt; *att = 0.0; }
    else { *a = 1.0; *at = 0.0; *att = 0.0; }
    return;
  }
  if (r.iramp == 33) {
    const double T_swtt = -log(0.1) / (10.0 * r.T_mono);
    *a = 1.0 - exp(-T_swtt * time);
    *at = (1.0 - *a) * T_swtt;
    *att = (1.0 - *a) * T_swtt * T_swtt;
    return;
  }
  if (time <= Tramp) {
    switch (r.iramp) {
      case 0: *a = 1.0; *at = 0.0; *att = 0.0; return;
      case 1: *a = time / Tramp; *at = 1.0 / Tramp; *att = 0.0; return;
      case 2: { const double t = time / Tramp; *a = t * t; *at = 2.0 * t / Tramp; *att = 2.0 / (Tramp * Tramp); return; }
      case 21: {
        const double T2 = Tramp * Tramp, tim2 = time * time, ts = time / Tramp - 1.0;
        if (time <= Tramp / 2.0) { *a = 2.0 * tim2 / T2; *at = 4.0 * time / T2; *att = 4.0 / T2; }
        else { *a = 1.0 - 2.0 * ts * ts; *at = -4.0 * ts / Tramp; *att = -4.0 / T2; }
        return;
      }
      case 4: { const double t = time / Tramp, t2 = t * t; *a = t2 * t2; *at = 4.0 * t2 * t / Tramp; *att = 12.0 * t2 / (Tramp * Tramp); return; }
      case 41: {
        const double T2 = Tramp * Tramp, tim2 = time * time, rap = 8.0 * time / Tramp, rap2 = tim2 / T2, rap22 = 3.0 * rap2;
        *a = (rap22 - rap + 6.0) * rap2; *at = (4.0 * rap22 - 3.0 * rap + 12.0) * time / T2; *att = (12.0 * rap22 - 6.0 * rap + 12.0) / T2;
        return;
      }
      default: return;  // unknown ramp: the reference leaves the values unchanged
    }
  }
  if (time >= r.T_stop + Tramp) { *a = 0.0; *at = 0.0; *att = 0.0; return; }
  if (time >= r.T_stop) {
    const double ti = r.T_stop + Tramp - time;
    switch (r.iramp) {
      case 1: *a = ti / Tramp; *at = -1.0 / Tramp; *att = 0.0; return;
      case 2: { const double t = ti / Tramp; *a = t * t; *at = -2.0 * t / Tramp; *att = 2.0 / (Tramp * Tramp); return; }
      case 21: {
        const double T2 = Tramp * Tramp, tim2 = ti * ti, ts = ti / Tramp - 1.0;
        if (ti <= Tramp / 2.0) { *a = 2.0 * tim2 / T2; *at = -4.0 * ti / T2; *att = 4.0 / T2; }
        else { *a = 1.0 - 2.0 * ts * ts; *at = 4.0 * ts / Tramp; *att = -4.0 / T2; }
        return;
      }
      case 4: { const double t = ti / Tramp, t2 = t * t; *a = t2 * t2; *at = -4.0 * t2 * t / Tramp; *att = 12.0 * t2 / (Tramp * Tramp); return; }
      case 41: {
        const double T2 = Tramp * Tramp, tim2 = ti * ti, rap = 8.0 * ti / Tramp, rap2 = tim2 / T2, rap22 = 3.0 * rap2;
        *a = (rap22 - rap + 6.0) * rap2; *at = -(4.0 * rap22 - 3.0 * rap + 12.0) * ti / T2; *att = (12.0 * rap22 - 6.0 * rap + 12.0) / T2;
        return;
      }
      default: return;
    }
  }
  *a = 1.0; *at = 0.0; *att = 0.0;
}

__global__ void k_eiwt(const double* __restrict__ freq, double* sc, double* eiwt, int nf, RampP rp) {
  pdl_wait();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n == 0) {
    // the wavemaker law of this stage (single writer of the ramp slots)
    double a = sc[SC_ALPHA], at = sc[SC_ALPHAT], att = sc[SC_ALPHATT];
    ramp_law(rp, sc[SC_TIME], &a, &at, &att);
    sc[SC_ALPHA] = a;
    sc[SC_ALPHAT] = at;
    sc[SC_ALPHATT] = att;
  }
  if (n >= nf) return;
  const double w = 6.283185307179586476925286766559005768394 * freq[n];
  double s, c;
  sincos(w * sc[SC_TIME], &s, &c);
  eiwt[2 * n] = c;
  eiwt[2 * n + 1] = s;
}

// pos_1st (wavemaking.f90:259-304) and the wavemaker boundary condition of
// SWEET_1 (resol_wmkr.f90:145-150).  One block per i2.
// mode 0: bc1 = -a*d2pos - 2 at*dpos - att*pos, bcr = -at*dpos - att*pos
// mode 1: bc1 = -a*dpos - at*pos (initial a1st_add, initial_condition.f90:388-392)
__global__ void k_pos_bc(const double* __restrict__ pos_re, const double* __restrict__ pos_im,
                         const double* __restrict__ freq, const double* __restrict__ eiwt,
                         const double* __restrict__ gzed, double* sc, int nf, int n2,
                         int n3, int n3a, double* bc1, double* bcr, int mode) {
  pdl_wait();
  const int i2 = blockIdx.x;
  const double a = sc[SC_ALPHA], at = sc[SC_ALPHAT], att = sc[SC_ALPHATT];
  double p0 = 0.0, p1 = 0.0, p2 = 0.0;
  for (int n = threadIdx.x; n < nf; n += blockDim.x) {
    const double w = 6.283185307179586476925286766559005768394 * freq[n];
    const double c = eiwt[2 * n], s = eiwt[2 * n + 1];
    const double pr = pos_re[i2 + (long long)n2 * n], pi = pos_im[i2 + (long long)n2 * n];
    const double rr = pr * c - pi * s;   // Re(pos * e^{iwt})
    const double ri = pr * s + pi * c;   // Im(pos * e^{iwt})
    p0 += rr;
    p1 += -ri * w;         // Re(resu * i w)
    p2 += -rr * w * w;     // Re(resu * (i w)^2)
  }
  p0 = block_reduce<0>(p0);
  __shared__ double P[3];
  if (threadIdx.x == 0) P[0] = p0;
  __syncthreads();
  p1 = block_reduce<0>(p1);
  if (threadIdx.x == 0) P[1] = p1;
  __syncthreads();
  p2 = block_reduce<0>(p2);
  if (threadIdx.x == 0) P[2] = p2;
  __syncthreads();
  for (int i3 = threadIdx.x; i3 < n3; i3 += blockDim.x) {
    const double g = gzed[i3];
    const double pos = g * P[0], dpos = g * P[1], d2pos = g * P[2];
    if (mode == 0) {
      bc1[i3 + (long long)n3a * i2] = -a * d2pos - 2.0 * at * dpos - att * pos;
      bcr[i3 + (long long)n3a * i2] = -at * dpos - att * pos;
    } else {
      bc1[i3 + (long long)n3a * i2] = -a * dpos - at * pos;
    }
  }
  if (i2 == 0 && threadIdx.x == 0) sc[SC_POSTOP] = gzed[n3 - 1] * P[0];
}

// match_surface_wmk (resol_wmkr.f90:1655-1741): rows n3..n3a-1 as a fixed
// linear combination of rows n3-4..n3-1 (the polynomial coefficients are
// linear in f, df, d2f).
__global__ void k_extend(double* a, double* b, const double* __restrict__ ext, int n2, int n3,
                         int n3a) {
  pdl_wait();
  const int nrow = n3a - n3;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int tot = nrow * n2;
  if (t >= 2 * tot) return;
  double* d = t < tot ? a : b;
  if (!d) return;
  const int u = t % tot;
  const int r = u % nrow, i2 = u / nrow;
  double* col = d + (long long)n3a * i2;
  const double* e = ext + 4 * r;
  col[n3 + r] = e[0] * col[n3 - 4] + e[1] * col[n3 - 3] + e[2] * col[n3 - 2] + e[3] * col[n3 - 1];
}

__global__ void k_div(double* a, double* b, const double* __restrict__ d, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  a[i] = a[i] / d[i];
  if (b) b[i] = b[i] / d[i];
}

// phiadd_1st_SWEET at z = 0 (resol_wmkr.f90:490-534), the i3 contraction:
// At(i1, j2) = sum_i3 da(i3,j2) cos(kx_add) csh;  Az(i1, j2) = -sum_i3 a(i3,j2) sin(kx_add) kx_add csh
// Block (16 x 8): 16 outputs i1, the i3 range split in 8 chunks, combined in
// shared memory in a fixed order.
constexpr int kCx = 16, kCy = 8;
__global__ void __launch_bounds__(kCx * kCy) k_sweet_contract(
    const double* __restrict__ a, const double* __restrict__ da, const double* __restrict__ cosk,
    const double* __restrict__ sink, const double* __restrict__ csh, const double* __restrict__ kxcsh,
    int n1, int n2, int n3a, double* At, double* Az) {
  pdl_wait();
  __shared__ double sa[512], sd[512];
  __shared__ double rt[kCy][kCx], rz[kCy][kCx];
  const int j2 = blockIdx.y;
  const int tx = threadIdx.x % kCx, ty = threadIdx.x / kCx;
  const int i1 = blockIdx.x * kCx + tx;
  for (int t = threadIdx.x; t < n3a; t += blockDim.x) {
    sa[t] = a[t + (long long)n3a * j2] * sink[t];
    sd[t] = da[t + (long long)n3a * j2] * cosk[t];
  }
  __syncthreads();
  const int ch = (n3a + kCy - 1) / kCy;
  double st = 0.0, sz = 0.0;
  if (i1 < n1) {
    for (int i3 = ty * ch; i3 < min(n3a, (ty + 1) * ch); ++i3) {
      const long long o = i1 + (long long)n1 * i3 + (long long)n1 * n3a * j2;
      st = fma(sd[i3], csh[o], st);
      sz = fma(sa[i3], kxcsh[o], sz);
    }
  }
  rt[ty][tx] = st;
  rz[ty][tx] = sz;
  __syncthreads();
  if (ty == 0 && i1 < n1) {
    double t = 0.0, z = 0.0;
    for (int c = 0; c < kCy; ++c) { t += rt[c][tx]; z += rz[c][tx]; }
    At[i1 + (long long)n1 * j2] = t;
    Az[i1 + (long long)n1 * j2] = -z;
  }
}

// SWEET_1 free-surface RHS (resol_wmkr.f90:177-185)
__global__ void k_sweet_rhs(const double* __restrict__ eta1st, const double* __restrict__ phit1,
                            const double* __restrict__ phiz1st_spec, const double* __restrict__ phiz1,
                            const double* __restrict__ nu, double iabsnb, double* rhs, double* keta1,
                            long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pz = phiz1st_spec[i] + phiz1[i];
  rhs[i] = -eta1st[i] - phit1[i] - iabsnb * nu[i] * pz;
  keta1[i] = pz;
}

// ---------------------------------------------------------------------------
// second-order wavemaker (i_wmk = 2)
// ---------------------------------------------------------------------------
// phiadd_1st_SWEET's free-surface set (resol_wmkr.f90:446-574) at z = 0,
// y-modal in j2 (the y sums follow as FOURIER_2_SPACE_y in 3-D tanks):
//   out_f(i1, j2) = s_f sum_i3 c_f(i3, j2) T_f(i1, j2, i3)
// with c_f one of a cos, da cos, a sin, da sin, a cos kx_add, a cos k_add^2,
// a sin kx_add, a sin ky (cos, sin of kx_add(i3)) and T_f one of csh,
// k_add sh, ky csh, kx_add csh.
enum { W_T = 0, W_Z, W_X, W_Y, W_ZZ, W_XT, W_YT, W_ZT, W_XX, W_XZ, W_YZ, W_NF };
struct Contract1Out {
  double* f[W_NF];
};
__global__ void __launch_bounds__(kCx * kCy) k_fs_contract1(
    const double* __restrict__ a, const double* __restrict__ da, const double* __restrict__ cosk,
    const double* __restrict__ sink, const double* __restrict__ kx_add, const double* __restrict__ k_add,
    const double* __restrict__ ky, const double* __restrict__ csh, const double* __restrict__ ksh,
    const double* __restrict__ kycsh, const double* __restrict__ kxcsh, int n1, int n2, int n3a,
    Contract1Out o) {
  pdl_wait();
  __shared__ double cf[8][512];
  __shared__ double red[W_NF][kCy][kCx];
  const int j2 = blockIdx.y;
  const int tx = threadIdx.x % kCx, ty = threadIdx.x / kCx;
  const int i1 = blockIdx.x * kCx + tx;
  for (int t = threadIdx.x; t < n3a; t += blockDim.x) {
    const double aa = a[t + (long long)n3a * j2], dd = da[t + (long long)n3a * j2];
    const double c = cosk[t], sn = sink[t], ka = k_add[t + (long long)n3a * j2];
    cf[0][t] = aa * c;
    cf[1][t] = dd * c;
    cf[2][t] = aa * sn;
    cf[3][t] = dd * sn;
    cf[4][t] = aa * c * kx_add[t];
    cf[5][t] = aa * c * (ka * ka);
    cf[6][t] = aa * sn * kx_add[t];
    cf[7][t] = aa * sn * ky[j2];
  }
  __syncthreads();
  const int ch = (n3a + kCy - 1) / kCy;
  double sm[W_NF];
#pragma unroll
  for (int f = 0; f < W_NF; ++f) sm[f] = 0.0;
  if (i1 < n1) {
    for (int i3 = ty * ch; i3 < min(n3a, (ty + 1) * ch); ++i3) {
      const long long q = i1 + (long long)n1 * i3 + (long long)n1 * n3a * j2;
      const double tc = csh[q], tk = ksh[q], ty_ = kycsh[q], tx_ = kxcsh[q];
      sm[W_T] = fma(cf[1][i3], tc, sm[W_T]);
      sm[W_Z] = fma(cf[2][i3], tx_, sm[W_Z]);
      sm[W_X] = fma(cf[0][i3], tk, sm[W_X]);
      sm[W_Y] = fma(cf[0][i3], ty_, sm[W_Y]);
      sm[W_ZZ] = fma(cf[4][i3], tx_, sm[W_ZZ]);
      sm[W_XT] = fma(cf[1][i3], tk, sm[W_XT]);
      sm[W_YT] = fma(cf[1][i3], ty_, sm[W_YT]);
      sm[W_ZT] = fma(cf[3][i3], tx_, sm[W_ZT]);
      sm[W_XX] = fma(cf[5][i3], tc, sm[W_XX]);
      sm[W_XZ] = fma(cf[6][i3], tk, sm[W_XZ]);
      sm[W_YZ] = fma(cf[7][i3], tc, sm[W_YZ]);
    }
  }
#pragma unroll
  for (int f = 0; f < W_NF; ++f) red[f][ty][tx] = sm[f];
  __syncthreads();
  if (ty == 0 && i1 < n1) {
    // signs of resol_wmkr.f90:500-532
    const double sg[W_NF] = {1.0, -1.0, -1.0, -1.0, -1.0, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0};
#pragma unroll
    for (int f = 0; f < W_NF; ++f) {
      double v = 0.0;
      for (int c = 0; c < kCy; ++c) v += red[f][c][tx];
      o.f[f][i1 + (long long)n1 * j2] = sg[f] * v;
    }
  }
}

// the wavemaker-grid terms of phiadd_1st_SWEET before their F2S_add
// (resol_wmkr.f90:536-543): a k_add^2, da k_add^2, -a ky, -da ky,
// -a kx_add, -da kx_add on the n3_add x n2 modes
struct AddProdOut {
  double* p[6];
};
__global__ void k_add_prod(const double* __restrict__ a, const double* __restrict__ da,
                           const double* __restrict__ k_add, const double* __restrict__ kx_add,
                           const double* __restrict__ ky, int n3a, long long n, AddProdOut o) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int i3 = (int)(i % n3a), i2 = (int)(i / n3a);
  const double aa = a[i], dd = da[i], ka = k_add[i];
  o.p[0][i] = aa * ka * ka;
  o.p[1][i] = dd * ka * ka;
  o.p[2][i] = -aa * ky[i2];
  o.p[3][i] = -dd * ky[i2];
  o.p[4][i] = -aa * kx_add[i3];
  o.p[5][i] = -dd * kx_add[i3];
}

// the free-surface mode products of d1st_for_2nd (resol_wmkr.f90:737-747)
// before their F2S: -a kx, -a ky, da kx, da ky, da kth1, -a kx^2, a k^2,
// -a kx kth1, (-a ky) kth1
struct FsProdOut {
  double* p[9];
};
__global__ void k_fs_prod1(const double* __restrict__ a, const double* __restrict__ da,
                           const double* __restrict__ kx, const double* __restrict__ ky,
                           const double* __restrict__ kth1, int n1, long long n, FsProdOut o) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int i1 = (int)(i % n1), i2 = (int)(i / n1);
  const double aa = a[i], dd = da[i], x = kx[i1], y = ky[i2], t = kth1[i];
  const double k = sqrt(x * x + y * y);
  o.p[0][i] = -aa * x;
  o.p[1][i] = -aa * y;
  o.p[2][i] = dd * x;
  o.p[3][i] = dd * y;
  o.p[4][i] = dd * t;
  o.p[5][i] = -aa * (x * x);
  o.p[6][i] = aa * k * k;
  o.p[7][i] = -aa * x * t;
  o.p[8][i] = (-aa * y) * t;
}

// d1st_for_2nd on the wavemaker (resol_wmkr.f90:703-717): the free-surface
// modes at the n3 wavemaker nodes, y-modal; one block per (i3, i2).
// out: -sum a T_xx, -sum da T_xx, -sum a T_y, -sum da T_y, sum a T_z, sum da T_z
struct WmkFsOut {
  double* w[6];
};
__global__ void k_wmk_from_fs(const double* __restrict__ a, const double* __restrict__ da,
                              const double* __restrict__ txx, const double* __restrict__ tyy,
                              const double* __restrict__ tz, int n1, int n2, int n3, WmkFsOut o) {
  pdl_wait();
  const int i3 = blockIdx.x, i2 = blockIdx.y;
  double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i1 = threadIdx.x; i1 < n1; i1 += blockDim.x) {
    const long long fi = i1 + (long long)n1 * i2;
    const long long q = fi + (long long)n1 * n2 * i3;
    const double aa = a[fi], dd = da[fi];
    s[0] = fma(aa, txx[q], s[0]);
    s[1] = fma(dd, txx[q], s[1]);
    s[2] = fma(aa, tyy[q], s[2]);
    s[3] = fma(dd, tyy[q], s[3]);
    s[4] = fma(aa, tz[q], s[4]);
    s[5] = fma(dd, tz[q], s[5]);
  }
  const double sg[6] = {-1.0, -1.0, -1.0, -1.0, 1.0, 1.0};
  for (int q = 0; q < 6; ++q) {
    const double v = block_reduce<0>(s[q]);
    if (threadIdx.x == 0) o.w[q][i3 + (long long)n3 * i2] = sg[q] * v;
    __syncthreads();
  }
}

// d1st_for_2nd on the free surface (resol_wmkr.f90:749-775): transformed
// products T (k_fs_prod1 order) plus the phiadd_1st_SWEET fields F
struct D1stArgs {
  const double* T[9];
  const double* F[W_NF];
  const double* phiz1st;  // F2S(a1st kth1)
  double* phix1st;
  double* phiy1st;
  double* etax1st;
  double* etay1st;
  double* phizt1st;
  double* phixx1st;
  double* phizz1st;
  double* phiz1st_tot;
};
__global__ void k_d1st_combine(D1stArgs g, const double* __restrict__ nu, const double* __restrict__ dnux,
                               double iabsnb, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pz = g.phiz1st[i] + g.F[W_Z][i];
  const double phixz = g.T[7][i] + g.F[W_XZ][i];
  const double phiyz = g.T[8][i] + g.F[W_YZ][i];
  g.phix1st[i] = g.T[0][i] + g.F[W_X][i];
  g.phiy1st[i] = g.T[1][i] + g.F[W_Y][i];
  g.etax1st[i] = g.T[2][i] - g.F[W_XT][i] - iabsnb * (dnux[i] * pz + nu[i] * phixz);
  g.etay1st[i] = g.T[3][i] - g.F[W_YT][i] - iabsnb * (0.0 * pz + nu[i] * phiyz);
  g.phizt1st[i] = g.T[4][i] + g.F[W_ZT][i];
  g.phixx1st[i] = g.T[5][i] + g.F[W_XX][i];
  g.phizz1st[i] = g.T[6][i] + g.F[W_ZZ][i];
  g.phiz1st_tot[i] = pz;
}

// solveHOS_SWEET_2's wavemaker condition (resol_wmkr.f90:262-281) with
// dposdy_1st / dposdz_1st (wavemaking.f90:313-406), no free-wave correction:
// one block per i2 sums the frequencies, then rows i3 < n3 of bc2.
// W: the six first-order wavemaker fields (wmk part n3 x n2, add part
// n3_add x n2, summed here).
struct Sweet2Wmk {
  const double* wf[6];  // k_wmk_from_fs outputs in space, n3 x n2
  const double* wa[6];  // F2S_add outputs, n3_add x n2
};
__global__ void k_sweet2_wmk(const double* __restrict__ pos_re, const double* __restrict__ pos_im,
                             const double* __restrict__ dy_re, const double* __restrict__ dy_im,
                             const double* __restrict__ freq, const double* __restrict__ eiwt,
                             const double* __restrict__ gzed, const double* __restrict__ dgzed,
                             const double* __restrict__ sc, int nf, int n2, int n3, int n3a, Sweet2Wmk W,
                             double* bc2) {
  pdl_wait();
  const int i2 = blockIdx.x;
  const double a = sc[SC_ALPHA], at = sc[SC_ALPHAT];
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int n = threadIdx.x; n < nf; n += blockDim.x) {
    const double w = 6.283185307179586476925286766559005768394 * freq[n];
    const double c = eiwt[2 * n], sn = eiwt[2 * n + 1];
    const long long q = i2 + (long long)n2 * n;
    const double pr = pos_re[q], pi = pos_im[q], yr = dy_re[q], yi = dy_im[q];
    s[0] += pr * c - pi * sn;            // Re(pos e^{iwt})
    s[1] += -(pr * sn + pi * c) * w;     // Re(pos e^{iwt} i w)
    s[2] += yr * c - yi * sn;            // Re(dposdy e^{iwt})
    s[3] += -(yr * sn + yi * c) * w;     // Re(dposdy e^{iwt} i w)
  }
  __shared__ double S[4];
  for (int q = 0; q < 4; ++q) {
    const double v = block_reduce<0>(s[q]);
    if (threadIdx.x == 0) S[q] = v;
    __syncthreads();
  }
  for (int i3 = threadIdx.x; i3 < n3; i3 += blockDim.x) {
    const double g = gzed[i3], dg = dgzed[i3];
    const double pos = g * S[0], dpos = g * S[1], dy = g * S[2], dyt = g * S[3], dz = dg * S[0], dzt = dg * S[1];
    const long long wi = i3 + (long long)n3 * i2, ai = i3 + (long long)n3a * i2;
    const double XX = W.wf[0][wi] + W.wa[0][ai], XXT = W.wf[1][wi] + W.wa[1][ai];
    const double Y = W.wf[2][wi] + W.wa[2][ai], YT = W.wf[3][wi] + W.wa[3][ai];
    const double Z = W.wf[4][wi] + W.wa[4][ai], ZT = W.wf[5][wi] + W.wa[5][ai];
    const double noramp = -pos * XX + dy * Y + dz * Z;
    bc2[ai] = -a * (-pos * XXT - dpos * XX + dy * YT + dyt * Y + dz * ZT + dzt * Z) - at * noramp;
  }
}

// solveHOS_SWEET_2's free-surface conditions (resol_wmkr.f90:301-312)
struct Sweet2Fs {
  const double* phiz2nd_spec;  // F2S(a2nd kth1)
  const double* p2z;
  const double* p2t;
  const double* eta2nd;
  const double* eta1st;
  const double* phix1st;
  const double* etax1st;
  const double* phiy1st;
  const double* etay1st;
  const double* phizz1st;
  const double* phiz1st;
  const double* phizt1st;
};
__global__ void k_sweet2_fs(Sweet2Fs g, const double* __restrict__ nu, double iabsnb, double* keta2,
                            double* rhs2, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pz2 = g.phiz2nd_spec[i] + g.p2z[i];
  const double px = g.phix1st[i], py = g.phiy1st[i], pz = g.phiz1st[i];
  const double deta = pz2 - px * g.etax1st[i] - py * g.etay1st[i] + g.eta1st[i] * g.phizz1st[i];
  keta2[i] = deta;
  rhs2[i] = -g.eta2nd[i] - g.p2t[i] - 5.0e-1 * (px * px + py * py + pz * pz) - g.eta1st[i] * g.phizt1st[i] -
            iabsnb * nu[i] * deta;
}

// the wavemaker-grid terms of wmk_3rdorder before their F2S_add
// (resol_wmkr.f90:962-981): first order -a k_add^2 kthk, -da k_add^2 kthk,
// a ky kthk, da ky kthk, a kx_add kthk, da kx_add kthk; second order
// a k_add^2, da k_add^2, -a ky, -da ky, -a kx_add, -da kx_add
struct AddProd3Out {
  double* p[12];
};
__global__ void k_add_prod3(const double* __restrict__ a1, const double* __restrict__ da1,
                            const double* __restrict__ a2, const double* __restrict__ da2,
                            const double* __restrict__ k_add, const double* __restrict__ kthk,
                            const double* __restrict__ kx_add, const double* __restrict__ ky, int n3a, long long n,
                            AddProd3Out o) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int i3 = (int)(i % n3a), i2 = (int)(i / n3a);
  const double ka = k_add[i], kt = kthk[i], y = ky[i2], x = kx_add[i3];
  const double aa = a1[i], dd = da1[i], bb = a2[i], ee = da2[i];
  o.p[0][i] = -aa * ka * ka * kt;
  o.p[1][i] = -dd * ka * ka * kt;
  o.p[2][i] = aa * y * kt;
  o.p[3][i] = dd * y * kt;
  o.p[4][i] = aa * x * kt;
  o.p[5][i] = dd * x * kt;
  o.p[6][i] = bb * ka * ka;
  o.p[7][i] = ee * ka * ka;
  o.p[8][i] = -bb * y;
  o.p[9][i] = -ee * y;
  o.p[10][i] = -bb * x;
  o.p[11][i] = -ee * x;
}

// solveHOS_SWEET_3's wavemaker condition (resol_wmkr.f90:370-397), no
// free-wave correction: one block per i2 sums the frequencies, then rows
// i3 < n3 of bc3.  X1: the six first-order fields (xxx, xxxt, xy, xyt, xz,
// xzt; F2S_add, n3_add x n2); X2: the six second-order fields (xx, xxt, y,
// yt, z, zt) as free-surface part (n3 x n2) plus F2S_add part.
struct Sweet3Wmk {
  const double* x1[6];
  const double* wf[6];
  const double* wa[6];
};
__global__ void k_sweet3_wmk(const double* __restrict__ pos_re, const double* __restrict__ pos_im,
                             const double* __restrict__ dy_re, const double* __restrict__ dy_im,
                             const double* __restrict__ freq, const double* __restrict__ eiwt,
                             const double* __restrict__ gzed, const double* __restrict__ dgzed,
                             const double* __restrict__ sc, int nf, int n2, int n3, int n3a, Sweet3Wmk W,
                             double* bc3) {
  pdl_wait();
  const int i2 = blockIdx.x;
  const double a = sc[SC_ALPHA], at = sc[SC_ALPHAT];
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int n = threadIdx.x; n < nf; n += blockDim.x) {
    const double w = 6.283185307179586476925286766559005768394 * freq[n];
    const double c = eiwt[2 * n], sn = eiwt[2 * n + 1];
    const long long q = i2 + (long long)n2 * n;
    const double pr = pos_re[q], pi = pos_im[q], yr = dy_re[q], yi = dy_im[q];
    s[0] += pr * c - pi * sn;
    s[1] += -(pr * sn + pi * c) * w;
    s[2] += yr * c - yi * sn;
    s[3] += -(yr * sn + yi * c) * w;
  }
  __shared__ double S[4];
  for (int q = 0; q < 4; ++q) {
    const double v = block_reduce<0>(s[q]);
    if (threadIdx.x == 0) S[q] = v;
    __syncthreads();
  }
  for (int i3 = threadIdx.x; i3 < n3; i3 += blockDim.x) {
    const double g = gzed[i3], dg = dgzed[i3];
    const double pos = g * S[0], dpos = g * S[1], dy = g * S[2], dyt = g * S[3], dz = dg * S[0], dzt = dg * S[1];
    const long long wi = i3 + (long long)n3 * i2, ai = i3 + (long long)n3a * i2;
    const double xxx = W.x1[0][ai], xxxt = W.x1[1][ai], xy = W.x1[2][ai], xyt = W.x1[3][ai];
    const double xz = W.x1[4][ai], xzt = W.x1[5][ai];
    const double xx2 = W.wf[0][wi] + W.wa[0][ai], xxt2 = W.wf[1][wi] + W.wa[1][ai];
    const double y2 = W.wf[2][wi] + W.wa[2][ai], yt2 = W.wf[3][wi] + W.wa[3][ai];
    const double z2 = W.wf[4][wi] + W.wa[4][ai], zt2 = W.wf[5][wi] + W.wa[5][ai];
    const double t_a = -a * (-dpos * xx2 - pos * xxt2 + dyt * y2 + dy * yt2 + dzt * z2 + dz * zt2);
    const double t_at = -at * (-pos * xx2 + dy * y2 + dz * z2);
    const double t_a2 = -(a * a) * (-(pos * pos) / 2.0 * xxxt - dpos * pos * xxx + dpos * dy * xy + pos * dy * xyt +
                                    pos * dyt * xy + dpos * dz * xz + pos * dz * xzt + pos * dzt * xz);
    const double t_aat = -a * at * (-(pos * pos) * xxx + 2.0 * pos * dy * xy + 2.0 * pos * dz * xz);
    bc3[ai] = t_a + t_at + t_a2 + t_aat;
  }
}

// phiadd_SL on a 1-D tank (n2 = 1): the i3 contraction at z = eta.
// kx_add(i3) = (2 i3 + 1) pi / 4, so cos/sin(kx_add(i3) (eta + 1)) follow
// from one sincos per chunk start and rotations by 2 phi, phi = pi (eta+1)/4.
__global__ void __launch_bounds__(kCx * kCy) k_phiadd_sl_1d(
    const double* __restrict__ eta, const double* __restrict__ a1, const double* __restrict__ a2,
    const double* __restrict__ a3, const double* __restrict__ da, const double* __restrict__ da2,
    const double* __restrict__ da3, const double* __restrict__ kx_add, const double* __restrict__ csh,
    const double* __restrict__ ksh,
    const double* __restrict__ kxcsh, int n1, int n3a, double* phix, double* phiy, double* phiz, double* phit,
    double* phi) {
  pdl_wait();
  __shared__ double sa[512], sd[512];
  __shared__ double r[4][kCy][kCx];
  const int tx = threadIdx.x % kCx, ty = threadIdx.x / kCx;
  const int i1 = blockIdx.x * kCx + tx;
  for (int t = threadIdx.x; t < n3a; t += blockDim.x) {
    sa[t] = a1[t] + a2[t] + a3[t];
    // da_add_1 + da_add_2 + da_add_3 (resol_HOS.f90:490)
    sd[t] = da3 ? da[t] + da2[t] + da3[t] : (da2 ? da[t] + da2[t] : da[t]);
  }
  __syncthreads();
  const int ch = (n3a + kCy - 1) / kCy;
  double st = 0.0, sx = 0.0, sz = 0.0, sp = 0.0;
  if (i1 < n1) {
    const double e1 = eta[i1] + 1.0;
    const int i3a = ty * ch, i3b = min(n3a, (ty + 1) * ch);
    if (i3a < i3b) {
      double s, c, s2, c2;
      sincos(kx_add[i3a] * e1, &s, &c);
      sincos(2.0 * kx_add[0] * e1, &s2, &c2);  // rotation by 2 phi
      for (int i3 = i3a; i3 < i3b; ++i3) {
        const long long o = i1 + (long long)n1 * i3;
        st = fma(sd[i3] * c, csh[o], st);
        sp = fma(sa[i3] * c, csh[o], sp);
        sx = fma(-sa[i3] * c, ksh[o], sx);
        sz = fma(-sa[i3] * s, kxcsh[o], sz);
        const double cn = c * c2 - s * s2;
        s = s * c2 + c * s2;
        c = cn;
      }
    }
  }
  r[0][ty][tx] = st;
  r[1][ty][tx] = sx;
  r[2][ty][tx] = sz;
  r[3][ty][tx] = sp;
  __syncthreads();
  if (ty == 0 && i1 < n1) {
    double t = 0.0, x = 0.0, z = 0.0, f = 0.0;
    for (int q = 0; q < kCy; ++q) { t += r[0][q][tx]; x += r[1][q][tx]; z += r[2][q][tx]; f += r[3][q][tx]; }
    phix[i1] = x;
    phiy[i1] = 0.0;
    phiz[i1] = z;
    phit[i1] = t;
    phi[i1] = f;
  }
}

// phiadd_SL (3-D): products Q_q(i1, i3, j2) = a(i3, j2) * T_q(i1, i3, j2)
__global__ void k_phiadd_q(const double* __restrict__ a1, const double* __restrict__ a2,
                           const double* __restrict__ a3, const double* __restrict__ da,
                           const double* __restrict__ da2, const double* __restrict__ da3,
                           const double* __restrict__ csh,
                           const double* __restrict__ ksh,
                           const double* __restrict__ kycsh, const double* __restrict__ kxcsh,
                           int n1, int n2, int n3a, double* Qt, double* Qx, double* Qy, double* Qz,
                           double* Qp) {
  pdl_wait();
  const long long n = (long long)n1 * n3a * n2;
  const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (o >= n) return;
  const long long r = o / n1;  // i3 + n3a * j2
  const double a = a1[r] + a2[r] + a3[r];
  Qt[o] = (da3 ? da[r] + da2[r] + da3[r] : (da2 ? da[r] + da2[r] : da[r])) * csh[o];
  Qx[o] = a * ksh[o];
  Qy[o] = a * kycsh[o];
  Qz[o] = a * kxcsh[o];
  Qp[o] = a * csh[o];
}

// phiadd_SL (3-D): contraction over i3 at z = eta of the y-transformed B_q
__global__ void k_phiadd_contract(const double* __restrict__ eta, const double* __restrict__ kx_add,
                                  const double* __restrict__ Bt, const double* __restrict__ Bx,
                                  const double* __restrict__ By, const double* __restrict__ Bz,
                                  const double* __restrict__ Bp, int n1, int n2, int n3a,
                                  double* phix, double* phiy, double* phiz, double* phit, double* phi) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)n1 * n2) return;
  const int i1 = (int)(i % n1), i2 = (int)(i / n1);
  const double e1 = eta[i] + 1.0;
  double st = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, sp = 0.0;
  for (int i3 = 0; i3 < n3a; ++i3) {
    double s, c;
    sincos(kx_add[i3] * e1, &s, &c);
    const long long o = i1 + (long long)n1 * i3 + (long long)n1 * n3a * i2;
    st += c * Bt[o];
    sx -= c * Bx[o];
    sy -= c * By[o];
    sz -= s * Bz[o];
    sp += c * Bp[o];
  }
  phix[i] = sx;
  phiy[i] = sy;
  phiz[i] = sz;
  phit[i] = st;
  phi[i] = sp;
}

// ---------------------------------------------------------------------------
// RK4(5) (runge_kutta.f90:81-360)
// ---------------------------------------------------------------------------
struct StageArgs {
  const double* k[4];
  double a[4];
  int nk;
  double c;
};
__global__ void k_rk_stage(const double* __restrict__ y0, StageArgs sa, double* sc, double* ys,
                           long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const double h = sc[SC_H];
  if (i < n) {
    double acc = 0.0;
    for (int t = 0; t < sa.nk; ++t) acc = acc + sa.k[t][i] * sa.a[t];
    ys[i] = y0[i] + h * acc;
  }
  if (i == 0) {
    sc[SC_TIME] = sc[SC_T0] + h * sa.c;
    sc[SC_DT] = h * sa.c;
  }
}

struct FinalArgs {
  const double* k[5];
  long long off[11];  // array boundaries of the state vector
};
// y_new = y0 + h sum b_j k_j; error estimate h (sum e_j k_j - sum b_j k_j),
// max |y_new| and max |erm| per array for the error norm (runge_kutta.f90:225-279)
__global__ void k_rk_final(const double* __restrict__ y0, FinalArgs fa, const double* __restrict__ sc,
                           double* ynew, double* part, long long n) {
  pdl_wait();
  const double h = sc[SC_H];
  const double b[5] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0.0};
  const double e[5] = {1.0 / 6.0, 2.0 / 3.0, 0.0, 0.0, 1.0 / 6.0};
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double mnew[5] = {0, 0, 0, 0, 0}, merr[5] = {0, 0, 0, 0, 0};
  if (i < n) {
    double db = 0.0, de = 0.0;
    for (int j = 0; j < 5; ++j) {
      const double kv = fa.k[j][i];
      db = db + kv * b[j];
      de = de + kv * e[j];
    }
    const double yn = y0[i] + h * db;
    ynew[i] = yn;
    int arr = 0;
    while (arr < 9 && i >= fa.off[arr + 1]) ++arr;
    // G1, G2, a_add_1, a_add_2, a_add_3 enter the error norm
    int slot = -1;
    if (arr == S_G1) slot = 0;
    else if (arr == S_G2) slot = 1;
    else if (arr == S_AADD1) slot = 2;
    else if (arr == S_AADD2) slot = 3;
    else if (arr == S_AADD3) slot = 4;
    if (slot >= 0) {
      mnew[slot] = fabs(yn);
      merr[slot] = fabs((de - db) * h);
    }
  }
  for (int s = 0; s < 5; ++s) {
    const double m1 = block_reduce<1>(mnew[s]);
    if (threadIdx.x == 0) part[blockIdx.x * 10 + s] = m1;
    const double m2 = block_reduce<1>(merr[s]);
    if (threadIdx.x == 0) part[blockIdx.x * 10 + 5 + s] = m2;
  }
}

__global__ void k_rk_err(const double* __restrict__ part, int nblocks, double* sc) {
  pdl_wait();
  // one block of 32 threads: max over blocks per slot, then the norm
  __shared__ double mx[10];
  if (threadIdx.x < 10) {
    double m = 0.0;
    for (int b = 0; b < nblocks; ++b) m = nan_max(m, part[b * 10 + threadIdx.x]);
    mx[threadIdx.x] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double tiny = 2.220446049250313080847263336181640625e-16;
    double err = 0.0;
    for (int s = 0; s < 5; ++s) err = nan_max(err, mx[5 + s] / (mx[s] + tiny));
    sc[SC_ERR] = err;
  }
}

// GtoF of the new state and of the stage-5 slope, phis/omega, deta and the
// volume correction (runge_kutta.f90:281-312)
__global__ void k_rk_out(const double* __restrict__ G1, const double* __restrict__ G2,
                         const double* __restrict__ k5G1, const double* __restrict__ k5G2,
                         const double* __restrict__ om, double* sc_, int n, int igeom,
                         double d_hinge, double xlen, double* etam, double* phim, double* detam,
                         double* part, unsigned int* counter) {
  pdl_wait();
  const double* sc = sc_;
  const double h = sc[SC_H];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < n) {
    const double w = om[i];
    double s, c;
    sincos(-w * h, &s, &c);
    const double g1 = G1[i], g2 = G2[i];
    e = g1 * c - g2 * s;
    double p = g2 * c + g1 * s;
    double d = k5G1[i] * c - k5G2[i] * s;
    if (i == 0) {
      p = sc[SC_PHIS0];
    } else {
      p = p / w;
      d = d + p * (w * w);
    }
    etam[i] = e;
    phim[i] = p;
    detam[i] = d;
  }
  const double bs = block_reduce<0>(e);
  if (threadIdx.x == 0) part[blockIdx.x] = bs;
  if (last_block(counter) && threadIdx.x == 0) {
    double S = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) S += __ldcg(part + b);
    volume_fix(etam, S, sc, igeom, d_hinge, xlen);
    *counter = 0;
  }
}

// G2 = S2F(phis) * omega, phisrk0 = S2F(phis)(1,1) (runge_kutta.f90:125-141)
__global__ void k_scale_omega(double* G2, const double* __restrict__ om, double* sc, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double g = G2[i];
  if (i == 0) sc[SC_PHIS0] = g;
  G2[i] = g * om[i];
}

__global__ void k_set_scalar(double* sc, int slot, double v) {
  pdl_wait(); sc[slot] = v; }

__global__ void k_sub(double* a, const double* __restrict__ b, long long n) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) a[i] -= b[i];
}

// probes: eta_p = sum S2F(eta) * mat_coscos (output.f90:265-282); one block per probe
__global__ void k_probe_dot(const double* __restrict__ modes, const double* __restrict__ mat,
                            long long n, double* out) {
  pdl_wait();
  const int p = blockIdx.x;
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += modes[i] * mat[n * p + i];
  s = block_reduce<0>(s);
  if (threadIdx.x == 0) out[p] = s;
}

// Diagnostics of one output time (single block, fixed order):
// out[0] = trapezoid sum of eta, out[1] of eta^2, out[2] of (phis + phi_add) deta
// (vol_energy.f90:36-119 before the mesh factors); out[3], out[4] = max |eta_x|,
// max |eta_y| on the dealiased grid (check_slope, initial_condition.f90:687-716).
__global__ void k_diagnostics(const double* __restrict__ eta, const double* __restrict__ phis,
                              const double* __restrict__ phi_add, const double* __restrict__ deta,
                              const double* __restrict__ etax, const double* __restrict__ etay, int n1,
                              int n2, long long nB, double* out) {
  pdl_wait();
  double v = 0.0, ep = 0.0, ek = 0.0, mx = 0.0, my = 0.0;
  const long long n = (long long)n1 * n2;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const int i1 = (int)(i % n1), i2 = (int)(i / n1);
    double w = (i1 == 0 || i1 == n1 - 1) ? 0.5 : 1.0;
    if (n2 != 1) w *= (i2 == 0 || i2 == n2 - 1) ? 0.5 : 1.0;
    const double e = eta[i];
    v += w * e;
    ep += w * (e * e);
    ek += w * ((phis[i] + phi_add[i]) * deta[i]);
  }
  for (long long i = threadIdx.x; i < nB; i += blockDim.x) {
    mx = nan_max(mx, fabs(etax[i]));
    my = nan_max(my, fabs(etay[i]));
  }
  v = block_reduce<0>(v);
  if (threadIdx.x == 0) out[0] = v;
  ep = block_reduce<0>(ep);
  if (threadIdx.x == 0) out[1] = ep;
  ek = block_reduce<0>(ek);
  if (threadIdx.x == 0) out[2] = ek;
  mx = block_reduce<1>(mx);
  if (threadIdx.x == 0) out[3] = mx;
  my = block_reduce<1>(my);
  if (threadIdx.x == 0) out[4] = my;
}

// zero the modes beyond nf along x (dir 0) or y (dir 1): the cut filter of
// filtering_base (filtering.f90:334-360)
__global__ void k_cut_modes(double* m, int n1, int n2, int nf, int dir) {
  pdl_wait();
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)n1 * n2) return;
  const int i1 = (int)(i % n1), i2 = (int)(i / n1);
  if ((dir == 0 && i1 >= nf) || (dir == 1 && i2 >= nf)) m[i] = 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------
// host-side orchestration
// ---------------------------------------------------------------------------
namespace {

struct Enq {
  Ctx& c;
  cudaStream_t st;
  const Params& P;
  const Dev& d;
  const Tables& tb;
  double* const* tmp;
  double* const* dt;  // temporaries of the truncated modes of dealiasing
  int ndt;
  Enq(Ctx& cc, cudaStream_t s)
      : c(cc), st(s), P(cc.P), d(cc.d), tb(cc.tb), tmp(cc.d.xtmp), dt(cc.d.dtmp), ndt(Dev::kDealiasTmp) {}
  Enq(Ctx& cc, cudaStream_t s, const Tables& t, double* const* tp, double* const* dtp, int nd)
      : c(cc), st(s), P(cc.P), d(cc.d), tb(t), tmp(tp), dt(dtp), ndt(nd) {}

  long long nN() const { return (long long)P.n1 * P.n2; }
  long long nB() const { return (long long)P.nd1 * P.nd2; }
  long long nA() const { return (long long)P.n3a * P.n2; }

  void xf(std::vector<XfReq> reqs) {
    for (size_t s = 0; s < reqs.size(); s += kMaxJobs) {
      const int cnt = (int)std::min<size_t>(kMaxJobs, reqs.size() - s);
      launch_transforms(reqs.data() + s, cnt, tb, tmp, st);
    }
  }
  XfReq R(int grid, int dir, int csx, int csy, const double* in, int in_ld, int nin1, int nin2,
          double* out, int out_ld, int nout1, int nout2, double scale = 1.0) const {
    XfReq r;
    r.grid = grid; r.dir = dir; r.csx = csx; r.csy = csy;
    r.in = in; r.in_ld = in_ld; r.nin1 = nin1; r.nin2 = nin2;
    r.out = out; r.out_ld = out_ld; r.nout1 = nout1; r.nout2 = nout2;
    r.scale = scale;
    return r;
  }
  // full-grid shorthands
  XfReq S2F_N(const double* in, double* out, int csx = 0, int csy = 0) const {
    return R(GRID_N, 1, csx, csy, in, P.n1, P.n1, P.n2, out, P.n1, P.n1, P.n2);
  }
  XfReq F2S_N(const double* in, double* out, int csx = 0, int csy = 0) const {
    return R(GRID_N, -1, csx, csy, in, P.n1, P.n1, P.n2, out, P.n1, P.n1, P.n2);
  }
  // F2S on the big grid of modes that are nonzero on e1 x e2 only (extend)
  XfReq F2S_B(const double* in, int in_ld, int e1, int e2, double* out, int csx = 0, int csy = 0) const {
    return R(GRID_BIG, -1, csx, csy, in, in_ld, e1, e2, out, P.nd1, P.nd1, P.nd2);
  }
  // the same request with its input multiplied by w[i1 + w_ld * i2]
  static XfReq weighted(XfReq r, const double* w, int w_ld) {
    r.win = w;
    r.win_ld = w_ld;
    return r;
  }
  bool act_x(int order) const { return P.p1 != 1 && (order - 1) % (P.p1 - 1) == 0; }
  bool act_y(int order) const { return P.n2 != 1 && P.p2 != 1 && (order - 1) % (P.p2 - 1) == 0; }
  bool dealias_on(int order) const { return act_x(order) || act_y(order); }
  int dclass(int order) const { return (act_x(order) ? 1 : 0) | (act_y(order) ? 2 : 0); }
  // dealias (dealiasing.f90:39-92): S2F_big, truncate, F2S_big, in place.
  // cls bit 0 truncates x to n1 modes, bit 1 truncates y to n2 modes; the
  // fields of one call are transformed together, ndt at a time.
  void dealias_many(const std::vector<std::pair<int, double*>>& fields) {
    std::vector<std::pair<int, double*>> f;
    for (const auto& p : fields)
      if (p.first != 0) f.push_back(p);
    for (size_t s = 0; s < f.size(); s += ndt) {
      const size_t e = std::min(f.size(), s + ndt);
      std::vector<XfReq> fw, bw;
      for (size_t i = s; i < e; ++i) {
        const int e1 = (f[i].first & 1) ? P.n1 : P.nd1, e2 = (f[i].first & 2) ? P.n2 : P.nd2;
        fw.push_back(R(GRID_BIG, 1, 0, 0, f[i].second, P.nd1, P.nd1, P.nd2, dt[i - s], P.nd1, e1, e2));
        bw.push_back(F2S_B(dt[i - s], P.nd1, e1, e2, f[i].second));
      }
      xf(fw);
      xf(bw);
    }
  }
  void dealias(int order, double* buf) {
    if (!dealias_on(order)) return;
    dealias_many({{dclass(order), buf}});
  }
  template <typename K, typename... A>
  void ew(K kern, long long n, A... a) {
    if (n <= 0) return;
    launch_pdl(kern, dim3(nblk(n)), dim3(kEW), 0, st, a...);
  }
  template <typename K, typename... A>
  void ew_trig(K kern, long long n, A... a) {
    if (n <= 0) return;
    launch_pdl(kern, dim3(nblk(n, kTrig)), dim3(kTrig), 0, st, a...);
  }
};

}  // namespace

void enqueue_set_scalar(Ctx& c, int slot, double v, cudaStream_t st) {
  launch_pdl(k_set_scalar, dim3(1), dim3(1), 0, st, c.d.sc, slot, v);
}

static RampP ramp_params(const Params& P) {
  RampP r;
  r.iramp = P.iramp;
  r.Tramp = P.Tramp;
  r.T_stop = P.T_stop;
  r.T_mono = P.T_mono;
  return r;
}

static bool has_wavemaker(const Params& P) {
  return P.icase != 1 && (P.igeom == 1 || P.igeom == 2);
}

// work fields of the second order in Dev::w2
enum {
  W2_F = 0,     // phiadd_1st_SWEET set in space (W_NF)
  W2_FM = 11,   // the same, y-modal (3-D tanks)
  W2_P9 = 22,   // free-surface products of d1st_for_2nd (9)
  W2_T9 = 31,   // their F2S (9)
  W2_AP = 40,   // wavemaker-grid products (6)
  W2_WA = 46,   // their F2S_add (6)
  W2_WFM = 52,  // free-surface modes on the wavemaker, y-modal (6)
  W2_WF = 58,   // the same in space (6)
  W2_PHIX = 64, W2_PHIY, W2_ETAX, W2_ETAY, W2_PHIZT, W2_PHIXX, W2_PHIZZ, W2_PZ,
  W2_BC2 = 72, W2_P2T, W2_P2Z, W2_P2TM, W2_P2ZM, W2_PZ2S, W2_RHS2, W2_A2K,
  W2_AP3 = 80,   // wavemaker-grid products of wmk_3rdorder (12)
  W2_WA3 = 92,   // their F2S_add (12)
  W2_WFM2 = 104, // second-order free-surface modes on the wavemaker, y-modal (6)
  W2_WF2 = 110,  // the same in space (6)
  W2_BC3 = 116,
  W2_COUNT
};
static_assert(W2_COUNT <= Dev::kW2, "second-order work fields");

// d1st_for_2nd and solveHOS_SWEET_2 (resol_wmkr.f90:219-329, 645-864) on the
// wavemaker stream, after solveHOS_SWEET_1 of the same stage: fills the
// slopes of a_add_2, a2nd and eta2nd.
void enqueue_sweet2(Ctx& c, Enq& W, const double* y, double* k) {
  const Params& P = c.P;
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const int n1 = P.n1, n2 = P.n2, n3 = P.n3, n3a = P.n3a;
  const long long nN = (long long)n1 * n2, nA = (long long)n3a * n2;
  cudaStream_t sw = W.st;
  const double* aA1 = y + L.off[S_AADD1];
  const double* kA1 = k + L.off[S_AADD1];
  const double* a1 = y + L.off[S_A1ST];
  const double* da1 = k + L.off[S_A1ST];
  double* const* w = d.w2;
  // wavemaker-grid terms of phiadd_1st_SWEET
  AddProdOut ap{};
  for (int q = 0; q < 6; ++q) ap.p[q] = w[W2_AP + q];
  W.ew(k_add_prod, nA, aA1, kA1, (const double*)d.k_add, (const double*)d.kx_add, (const double*)d.ky, n3a,
       nA, ap);
  {
    std::vector<XfReq> rq;
    const int kz[6] = {0, 0, 0, 0, 1, 1}, ky_[6] = {0, 0, 1, 1, 0, 0};
    for (int q = 0; q < 6; ++q)
      rq.push_back(W.R(GRID_ADD, -1, kz[q], ky_[q], w[W2_AP + q], n3a, n3a, n2, w[W2_WA + q], n3a, n3a, n2));
    W.xf(rq);
  }
  // d1st_for_2nd on the free surface: products and their F2S
  FsProdOut fp{};
  for (int q = 0; q < 9; ++q) fp.p[q] = w[W2_P9 + q];
  W.ew(k_fs_prod1, nN, a1, da1, (const double*)d.kx, (const double*)d.ky, (const double*)d.kth1, n1, nN, fp);
  {
    std::vector<XfReq> rq;
    const int kx_[9] = {1, 0, 1, 0, 0, 0, 0, 1, 0}, ky_[9] = {0, 1, 0, 1, 0, 0, 0, 0, 1};
    for (int q = 0; q < 9; ++q) rq.push_back(W.F2S_N(w[W2_P9 + q], w[W2_T9 + q], kx_[q], ky_[q]));
    W.xf(rq);
  }
  // d1st_for_2nd on the wavemaker
  WmkFsOut wo{};
  for (int q = 0; q < 6; ++q) wo.w[q] = n2 == 1 ? w[W2_WF + q] : w[W2_WFM + q];
  launch_pdl(k_wmk_from_fs, dim3(n3, n2), dim3(128), 0, sw, a1, da1, (const double*)d.kx2cshx,
             (const double*)d.kycshx, (const double*)d.kshx, n1, n2, n3, wo);
  if (n2 != 1)
    for (int q = 0; q < 6; ++q)
      launch_y_f2s(W.tb, w[W2_WFM + q], n3, n3, w[W2_WF + q], n3, (q == 2 || q == 3) ? 1 : 0, sw);
  D1stArgs g{};
  for (int q = 0; q < 9; ++q) g.T[q] = w[W2_T9 + q];
  for (int f = 0; f < W_NF; ++f) g.F[f] = w[W2_F + f];
  g.phiz1st = d.phiz1st;
  g.phix1st = w[W2_PHIX];
  g.phiy1st = w[W2_PHIY];
  g.etax1st = w[W2_ETAX];
  g.etay1st = w[W2_ETAY];
  g.phizt1st = w[W2_PHIZT];
  g.phixx1st = w[W2_PHIXX];
  g.phizz1st = w[W2_PHIZZ];
  g.phiz1st_tot = w[W2_PZ];
  W.ew(k_d1st_combine, nN, g, (const double*)d.nu, (const double*)d.dnux, (double)P.iabsnb, nN);
  // the second-order wavemaker condition, matched, transformed, divided
  Sweet2Wmk sv{};
  for (int q = 0; q < 6; ++q) {
    sv.wf[q] = w[W2_WF + q];
    sv.wa[q] = w[W2_WA + q];
  }
  launch_pdl(k_sweet2_wmk, dim3(n2), dim3(128), 0, sw, (const double*)d.pos_re, (const double*)d.pos_im,
             (const double*)d.dposdy_re, (const double*)d.dposdy_im, (const double*)d.freq_w,
             (const double*)d.eiwt, (const double*)d.gzed, (const double*)d.dgzed, (const double*)d.sc, c.nf, n2,
             n3, n3a, sv, w[W2_BC2]);
  {
    const int tot = (n3a - n3) * n2;
    launch_pdl(k_extend, dim3(nblk(tot)), dim3(kEW), 0, sw, w[W2_BC2], (double*)nullptr, d.ext, n2, n3, n3a);
  }
  double* kA2 = k + L.off[S_AADD2];
  W.xf({W.R(GRID_ADD, 1, 0, 0, w[W2_BC2], n3a, n3a, n2, kA2, n3a, n3a, n2)});
  W.ew(k_div, nA, kA2, (double*)nullptr, (const double*)d.k_add_thk, nA);
  // phiadd_2nd: phit_add_2, phiz_add_2 at z = 0
  const double* aA2 = y + L.off[S_AADD2];
  launch_pdl(k_sweet_contract, dim3((n1 + kCx - 1) / kCx, n2), dim3(kCx * kCy), 0, sw, aA2,
             (const double*)kA2, (const double*)d.cosk, (const double*)d.sink, (const double*)d.csh,
             (const double*)d.kxcsh, n1, n2, n3a, n2 == 1 ? w[W2_P2T] : w[W2_P2TM],
             n2 == 1 ? w[W2_P2Z] : w[W2_P2ZM]);
  if (n2 != 1) {
    launch_y_f2s(W.tb, w[W2_P2TM], n1, n1, w[W2_P2T], n1, 0, sw);
    launch_y_f2s(W.tb, w[W2_P2ZM], n1, n1, w[W2_P2Z], n1, 0, sw);
  }
  // phidphiz of the second order and the free-surface conditions
  W.ew(k_mul, nN, y + L.off[S_A2ND], (const double*)d.kth1, 1.0, w[W2_A2K], nN);
  W.xf({W.F2S_N(w[W2_A2K], w[W2_PZ2S])});
  Sweet2Fs fs{};
  fs.phiz2nd_spec = w[W2_PZ2S];
  fs.p2z = w[W2_P2Z];
  fs.p2t = w[W2_P2T];
  fs.eta2nd = y + L.off[S_ETA2ND];
  fs.eta1st = y + L.off[S_ETA1ST];
  fs.phix1st = w[W2_PHIX];
  fs.etax1st = w[W2_ETAX];
  fs.phiy1st = w[W2_PHIY];
  fs.etay1st = w[W2_ETAY];
  fs.phizz1st = w[W2_PHIZZ];
  fs.phiz1st = w[W2_PZ];
  fs.phizt1st = w[W2_PHIZT];
  W.ew(k_sweet2_fs, nN, fs, (const double*)d.nu, (double)P.iabsnb, k + L.off[S_ETA2ND], w[W2_RHS2], nN);
  W.xf({W.S2F_N(w[W2_RHS2], k + L.off[S_A2ND])});
}

// wmk_3rdorder and solveHOS_SWEET_3 (resol_wmkr.f90:338-437, 942-1115) on
// the wavemaker stream after enqueue_sweet2: fills the slope of a_add_3.
void enqueue_sweet3(Ctx& c, Enq& W, const double* y, double* k) {
  const Params& P = c.P;
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const int n1 = P.n1, n2 = P.n2, n3 = P.n3, n3a = P.n3a;
  const long long nA = (long long)n3a * n2;
  cudaStream_t sw = W.st;
  double* const* w = d.w2;
  AddProd3Out ap{};
  for (int q = 0; q < 12; ++q) ap.p[q] = w[W2_AP3 + q];
  W.ew(k_add_prod3, nA, y + L.off[S_AADD1], (const double*)(k + L.off[S_AADD1]), y + L.off[S_AADD2],
       (const double*)(k + L.off[S_AADD2]), (const double*)d.k_add, (const double*)d.k_add_thk,
       (const double*)d.kx_add, (const double*)d.ky, n3a, nA, ap);
  {
    std::vector<XfReq> rq;
    for (int q = 0; q < 12; ++q) {
      const int kind = q % 6;  // cos,cos (0,1) cos,sin (2,3) sin,cos (4,5)
      rq.push_back(W.R(GRID_ADD, -1, kind >= 4 ? 1 : 0, (kind == 2 || kind == 3) ? 1 : 0, w[W2_AP3 + q], n3a, n3a,
                       n2, w[W2_WA3 + q], n3a, n3a, n2));
    }
    W.xf(rq);
  }
  WmkFsOut wo{};
  for (int q = 0; q < 6; ++q) wo.w[q] = n2 == 1 ? w[W2_WF2 + q] : w[W2_WFM2 + q];
  launch_pdl(k_wmk_from_fs, dim3(n3, n2), dim3(128), 0, sw, y + L.off[S_A2ND], (const double*)(k + L.off[S_A2ND]),
             (const double*)d.kx2cshx, (const double*)d.kycshx, (const double*)d.kshx, n1, n2, n3, wo);
  if (n2 != 1)
    for (int q = 0; q < 6; ++q)
      launch_y_f2s(W.tb, w[W2_WFM2 + q], n3, n3, w[W2_WF2 + q], n3, (q == 2 || q == 3) ? 1 : 0, sw);
  Sweet3Wmk sv{};
  for (int q = 0; q < 6; ++q) {
    sv.x1[q] = w[W2_WA3 + q];
    sv.wf[q] = w[W2_WF2 + q];
    sv.wa[q] = w[W2_WA3 + 6 + q];
  }
  launch_pdl(k_sweet3_wmk, dim3(n2), dim3(128), 0, sw, (const double*)d.pos_re, (const double*)d.pos_im,
             (const double*)d.dposdy_re, (const double*)d.dposdy_im, (const double*)d.freq_w,
             (const double*)d.eiwt, (const double*)d.gzed, (const double*)d.dgzed, (const double*)d.sc, c.nf, n2,
             n3, n3a, sv, w[W2_BC3]);
  {
    const int tot = (n3a - n3) * n2;
    launch_pdl(k_extend, dim3(nblk(tot)), dim3(kEW), 0, sw, w[W2_BC3], (double*)nullptr, d.ext, n2, n3, n3a);
  }
  double* kA3 = k + L.off[S_AADD3];
  W.xf({W.R(GRID_ADD, 1, 0, 0, w[W2_BC3], n3a, n3a, n2, kA3, n3a, n3a, n2)});
  W.ew(k_div, nA, kA3, (double*)nullptr, (const double*)d.k_add_thk, nA);
}

void enqueue_rhs(Ctx& c, const double* y, double* k, bool rk_mode, cudaStream_t st) {
  Enq E(c, st);
  const Params& P = c.P;
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const int n1 = P.n1, n2 = P.n2, nd1 = P.nd1, nd2 = P.nd2, M = P.M;
  const long long nN = E.nN(), nB = E.nB(), nA = E.nA();
  const double* G1 = y + L.off[S_G1];
  const double* G2 = y + L.off[S_G2];
  double* kG1 = k + L.off[S_G1];
  double* kG2 = k + L.off[S_G2];
  c.n_rhs++;

  // 1. GtoF + volume correction of the mean mode
  {
    const int nb = nblk(nN, kTrig);
    launch_pdl(k_gtof, dim3(nb), dim3(kTrig), 0, st, G1, G2, d.omega, d.kx, d.ky, d.sc, n1, n2, P.igeom, P.d_hinge,
                               P.xlen, d.etam, d.phim, d.w_eta_x, d.w_eta_y, d.w_phi_x, d.w_phi_y,
                               d.part, d.counter);
  }
  // 5. wavemaker: SWEET_1, phiadd_SL and the gradients of phi_add.  This
  //    branch reads the free surface only through eta in space, so it runs
  //    on the second stream with its own transform scratch and joins the
  //    main stream before assembly.
  cudaStream_t sw = c.st2;
  Enq W(c, sw, c.tb2, d.xtmp2, nullptr, 0);
  const bool wmk2 = has_wavemaker(P) && P.i_wmk >= 2;
  const bool wmk3 = has_wavemaker(P) && P.i_wmk == 3;
  cudaEventRecord(c.ev_fork, st);
  cudaStreamWaitEvent(sw, c.ev_fork, 0);
  double* kA1 = k + L.off[S_AADD1];
  double* kAR = k + L.off[S_AADDR];
  double* kA1st = k + L.off[S_A1ST];
  double* kEta1 = k + L.off[S_ETA1ST];
  if (has_wavemaker(P)) {
    const RampP rp = ramp_params(P);
    launch_pdl(k_eiwt, dim3(nblk(c.nf > 0 ? c.nf : 1)), dim3(kEW), 0, sw, d.freq_w, d.sc, d.eiwt, c.nf, rp);
    launch_pdl(k_pos_bc, dim3(n2), dim3(128), 0, sw, d.pos_re, d.pos_im, d.freq_w, d.eiwt, d.gzed, d.sc, c.nf, n2,
                                 P.n3, P.n3a, d.bc1, d.bcr, 0);
    {
      const int tot = 2 * (P.n3a - P.n3) * n2;
      launch_pdl(k_extend, dim3(nblk(tot)), dim3(kEW), 0, sw, d.bc1, d.bcr, d.ext, n2, P.n3, P.n3a);
    }
    W.xf({W.R(GRID_ADD, 1, 0, 0, d.bc1, P.n3a, P.n3a, n2, kA1, P.n3a, P.n3a, n2),
          W.R(GRID_ADD, 1, 0, 0, d.bcr, P.n3a, P.n3a, n2, kAR, P.n3a, P.n3a, n2)});
    W.ew(k_div, nA, kA1, kAR, (const double*)d.k_add_thk, nA);
    // reconstruction at z = 0 (phiadd_1st_SWEET) for phit_add_1, phiz_add_1
    const double* aA1 = y + L.off[S_AADD1];
    const double* phit1 = d.phit_add1;
    const double* phiz1 = d.phiz_add1;
    if (wmk2) {
      // the whole first-order set that the second order needs
      Contract1Out co{};
      for (int f = 0; f < W_NF; ++f) co.f[f] = n2 == 1 ? d.w2[W2_F + f] : d.w2[W2_FM + f];
      launch_pdl(k_fs_contract1, dim3((n1 + kCx - 1) / kCx, n2), dim3(kCx * kCy), 0, sw, aA1,
                 (const double*)kA1, (const double*)d.cosk, (const double*)d.sink, (const double*)d.kx_add,
                 (const double*)d.k_add, (const double*)d.ky, (const double*)d.csh, (const double*)d.ksh,
                 (const double*)d.kycsh, (const double*)d.kxcsh, n1, n2, P.n3a, co);
      if (n2 != 1)
        for (int f = 0; f < W_NF; ++f)
          launch_y_f2s(W.tb, d.w2[W2_FM + f], n1, n1, d.w2[W2_F + f], n1,
                       (f == W_Y || f == W_YT || f == W_YZ) ? 1 : 0, sw);
      phit1 = d.w2[W2_F + W_T];
      phiz1 = d.w2[W2_F + W_Z];
    } else {
      launch_pdl(k_sweet_contract, dim3(dim3((n1 + kCx - 1) / kCx, n2)), dim3(kCx * kCy), 0, sw,
          aA1, kA1, d.cosk, d.sink, d.csh, d.kxcsh, n1, n2, P.n3a, n2 == 1 ? d.phit_add1 : d.Q[0],
          n2 == 1 ? d.phiz_add1 : d.Q[1]);
      if (n2 != 1) {
        // y sums: sum_j2 A(i1, j2) cos(ky(j2) y(i2)) = FOURIER_2_SPACE_y
        launch_y_f2s(W.tb, d.Q[0], n1, n1, d.phit_add1, n1, 0, sw);
        launch_y_f2s(W.tb, d.Q[1], n1, n1, d.phiz_add1, n1, 0, sw);
      }
    }
    // phidphiz + SWEET_1 RHS
    W.ew(k_mul, nN, y + L.off[S_A1ST], (const double*)d.kth1, 1.0, d.a1k, nN);
    W.xf({W.F2S_N(d.a1k, d.phiz1st)});
    W.ew(k_sweet_rhs, nN, y + L.off[S_ETA1ST], phit1, (const double*)d.phiz1st, phiz1,
         (const double*)d.nu, (double)P.iabsnb, d.rhs1, kEta1, nN);
    W.xf({W.S2F_N(d.rhs1, kA1st)});
    if (wmk2) enqueue_sweet2(c, W, y, k);
    if (wmk3) enqueue_sweet3(c, W, y, k);
  }
  // Slopes of the wavemaker arrays that this tank never forms (no wavemaker;
  // orders above i_wmk) stay zero: the slope buffers are zero-filled when
  // they are allocated and only the branches above write those parts.

  // 2. transform batch A: eta in space, eta / eta_x / eta_y / phis_x / phis_y on
  //    the big grid (phisxy_etaxy) and the order-1 HOS terms F2S_big(a1 kth_ext(j))
  {
    std::vector<XfReq> rq;
    rq.push_back(E.F2S_N(d.etam, d.eta_sp));
    rq.push_back(E.F2S_B(d.etam, n1, n1, n2, d.etapm[0]));
    rq.push_back(E.F2S_B(d.w_eta_x, n1, n1, n2, d.etax, 1, 0));
    rq.push_back(E.F2S_B(d.w_phi_x, n1, n1, n2, d.phisx, 1, 0));
    if (n2 != 1) {
      rq.push_back(E.F2S_B(d.w_eta_y, n1, n1, n2, d.etay, 0, 1));
      rq.push_back(E.F2S_B(d.w_phi_y, n1, n1, n2, d.phisy, 0, 1));
    }
    // F2S_big(phis_modes * kth_ext(j)): the products are taken as the
    // transform reads its input
    for (int j = 1; j <= M; ++j)
      rq.push_back(E.weighted(E.F2S_B(d.phim, n1, n1, n2, d.phizi[(0) * M + (j - 1)]),
                              d.kth_ext + (long long)nd1 * nd2 * (j - 1), nd1));
    E.xf(rq);
    cudaEventRecord(c.ev_eta, st);
    // in 2-D tanks eta_y and phis_y stay zero: their buffers are zero-filled
    // when allocated and only the y-gradient transforms above write them
  }
  // 5b. wavemaker branch, second part: phiadd_SL with the total additional
  //     amplitudes at z = eta (needs eta in space from batch A) and the
  //     gradients of phi_add on the big grid (resol_HOS.f90:534-555)
  if (has_wavemaker(P)) {
    const double* kA2 = wmk2 ? k + L.off[S_AADD2] : nullptr;
    const double* kA3 = wmk3 ? k + L.off[S_AADD3] : nullptr;
    cudaStreamWaitEvent(sw, c.ev_eta, 0);
    const double* aA1 = y + L.off[S_AADD1];
    const double* aA2 = y + L.off[S_AADD2];
    const double* aA3 = y + L.off[S_AADD3];
    if (n2 == 1) {
      launch_pdl(k_phiadd_sl_1d, dim3((n1 + kCx - 1) / kCx), dim3(kCx * kCy), 0, sw, d.eta_sp, aA1, aA2,
                 aA3, (const double*)kA1, kA2, kA3, d.kx_add, d.csh, d.ksh, d.kxcsh, n1, P.n3a, d.phix_add,
                 d.phiy_add, d.phiz_add, d.phit_add, d.phi_add);
    } else {
      const long long nq = (long long)n1 * P.n3a * n2;
      W.ew(k_phiadd_q, nq, aA1, aA2, aA3, (const double*)kA1, kA2, kA3, (const double*)d.csh,
           (const double*)d.ksh, (const double*)d.kycsh, (const double*)d.kxcsh, n1, n2, P.n3a,
           d.Q[0], d.Q[1], d.Q[2], d.Q[3], d.Q[4]);
      const int lines = n1 * P.n3a;
      launch_y_f2s(W.tb, d.Q[0], lines, lines, d.B[0], lines, 0, sw);
      launch_y_f2s(W.tb, d.Q[1], lines, lines, d.B[1], lines, 0, sw);
      launch_y_f2s(W.tb, d.Q[2], lines, lines, d.B[2], lines, 1, sw);
      launch_y_f2s(W.tb, d.Q[3], lines, lines, d.B[3], lines, 0, sw);
      launch_y_f2s(W.tb, d.Q[4], lines, lines, d.B[4], lines, 0, sw);
      W.ew(k_phiadd_contract, nN, (const double*)d.eta_sp, (const double*)d.kx_add,
           (const double*)d.B[0], (const double*)d.B[1], (const double*)d.B[2],
           (const double*)d.B[3], (const double*)d.B[4], n1, n2, P.n3a, d.phix_add, d.phiy_add,
           d.phiz_add, d.phit_add, d.phi_add);
    }
  }
  // without a wavemaker phi_add and its derivatives stay zero (zero-filled
  // at allocation, written only by the phiadd_SL kernels above)
  W.xf({W.S2F_N(d.phix_add, d.pmode[0]), W.S2F_N(d.phiy_add, d.pmode[1]),
        W.S2F_N(d.phiz_add, d.pmode[2])});
  W.xf({W.F2S_B(d.pmode[0], n1, n1, n2, d.pxe), W.F2S_B(d.pmode[1], n1, n1, n2, d.pye),
        W.F2S_B(d.pmode[2], n1, n1, n2, d.pze)});
  cudaEventRecord(c.ev_join, sw);
  // event after which eta^o/o! is final (orders >= 2), -1: the full join
  std::vector<int> pw_ev(M + 2, -1);
  int npw = 0;
  // 3. powers eta^j / j! with partial dealiasing (one kernel per run of
  //    orders up to the next order that is dealiased) and |grad eta|^2.
  //    Order 1 of the HOS recursion needs none of them, so they run on a
  //    third stream and join before order 2.
  {
    cudaStream_t sp = c.st3;
    Enq Pw(c, sp, c.tb3, d.xtmp3, &d.ptmp, 1);
    cudaStreamWaitEvent(sp, c.ev_eta, 0);
    for (int j = 1; j < M;) {
      int jend = j + 1;
      while (jend < M && !E.dealias_on(jend)) ++jend;
      PowArgs pa{};
      for (int t = 0; t < M; ++t) pa.e[t] = d.etapm[t];
      pa.j0 = j;
      pa.j1 = jend;
      Pw.ew(k_pow_run, nB, pa, nB);
      // orders j+1 .. jend are final here, except jend when it is dealiased
      const bool dl_end = E.dealias_on(jend);
      if (npw < Ctx::kPowEvents) {
        cudaEventRecord(c.ev_pw[npw], sp);
        for (int o = j + 1; o <= jend - (dl_end ? 1 : 0); ++o) pw_ev[o] = npw;
        ++npw;
      }
      if (dl_end) {
        Pw.dealias(jend, d.etapm[jend - 1]);
        if (npw < Ctx::kPowEvents) {
          cudaEventRecord(c.ev_pw[npw], sp);
          pw_ev[jend] = npw++;
        }
      }
      j = jend;
    }
    Pw.ew(k_sq2, nB, (const double*)d.etax, (const double*)d.etay, d.gradeta2, nB);
    Pw.dealias(2, d.gradeta2);
    cudaEventRecord(c.ev_pow, sp);
  }
  bool pow_joined = false;
  // Dealiasing of phizm(iHOS): the recursion goes on with the undealiased
  // phimext, so intermediate orders are dealiased on the third stream (joined
  // before the quadratic products) and the last order, which only the
  // assembly reads, joins the batch after the products.
  std::vector<std::pair<int, double*>> dl_late;
  bool side_dealias = false;

  // 4. HOS recursion (HOSphis_modes)
  std::vector<int> ext1(M + 2, nd1), ext2(M + 2, nd2);
  // In 3-D tanks, orders 2 .. kAccMax are accumulated by the final pass of
  // the F2S batch that produces their first term (AccEpi), which saves a
  // pass over the big grid per order; order 1 follows batch A, which also
  // produces eta, so it keeps its own kernel.  In 2-D tanks the separate
  // kernel is cheaper than the epilogue's dependent loads.
  const bool fuse_acc = (n2 > 1);
  auto join_pow = [&]() {
    if (!pow_joined) {
      cudaStreamWaitEvent(st, c.ev_pow, 0);
      pow_joined = true;
    }
  };
  // wait until eta^j/j! is final for every j <= o
  int pw_waited = -1;
  auto wait_powers = [&](int o) {
    for (int q = 2; q <= o; ++q)
      if (pw_ev[q] < 0) {
        join_pow();
        return;
      }
    if (pow_joined || o < 2) return;
    const int idx = pw_ev[o];
    if (idx > pw_waited) {
      cudaStreamWaitEvent(st, c.ev_pw[idx], 0);
      pw_waited = idx;
    }
  };
  std::vector<AccEpi> epis(M + 2);
  for (int iHOS = 1; iHOS <= M; ++iHOS) {
    if (iHOS == 1 || iHOS > kAccMax || !fuse_acc) {
      wait_powers(iHOS);
      AccArgs aa{};
      aa.iHOS = iHOS;
      for (int j = 1; j <= iHOS; ++j) {
        const int m = iHOS + 1 - j;
        aa.phizi[j - 1] = d.phizi[(m - 1) * M + (j - 1)];
        aa.etapm[j - 1] = d.etapm[j - 1];
      }
      E.ew(k_hos_accum, nB, aa, d.phimext, d.phizm[iHOS], nB);
    }
    if (iHOS > 1 && E.dealias_on(iHOS)) {
      if (iHOS == M) {
        dl_late.push_back({E.dclass(M), d.phizm[M]});
      } else {
        cudaEventRecord(c.ev_acc, st);
        cudaStreamWaitEvent(c.st3, c.ev_acc, 0);
        Enq Pd(c, c.st3, c.tb3, d.xtmp3, &d.ptmp, 1);
        Pd.dealias(iHOS, d.phizm[iHOS]);
        side_dealias = true;
      }
    }
    if (iHOS < M) {
      const int o = iHOS + 1;
      const int e1 = E.act_x(o) ? n1 : nd1;
      const int e2 = E.act_y(o) ? n2 : nd2;
      ext1[o] = e1;
      ext2[o] = e2;
      E.xf({E.R(GRID_BIG, 1, 0, 0, d.phimext, nd1, nd1, nd2, d.aHOS[o], nd1, e1, e2)});
      // F2S_big of the products with kth_ext(j), j = 1 .. M+1-o
      std::vector<XfReq> rq;
      for (int j = 1; j <= M + 1 - o; ++j)
        rq.push_back(E.weighted(E.F2S_B(d.aHOS[o], nd1, e1, e2, d.phizi[(o - 1) * M + (j - 1)]),
                                d.kth_ext + (long long)nd1 * nd2 * (j - 1), nd1));
      if (fuse_acc && o <= kAccMax) {
        // order o's accumulation on the outputs of its first term, phizi(o, 1)
        AccEpi& ae = epis[o];
        ae.iHOS = o;
        for (int j = 1; j <= o; ++j) {
          ae.z[j - 1] = d.phizi[(o - j) * M + (j - 1)];
          ae.e[j - 1] = d.etapm[j - 1];
        }
        ae.phimext = d.phimext;
        ae.phizm = d.phizm[o];
        rq[0].acc = &ae;
        wait_powers(o);
      }
      E.xf(rq);
    }
  }
  if (!pow_joined) cudaStreamWaitEvent(st, c.ev_pow, 0);
  if (side_dealias) {
    cudaEventRecord(c.ev_dl, c.st3);
    cudaStreamWaitEvent(st, c.ev_dl, 0);
  }
  // Quadratic terms of HOSphis_modes (resol_HOS.f90:797-905): every term is
  // dealiased at its order; dealiasing is linear, so terms are summed per
  // dealiasing class first (class = which directions the order truncates).
  struct Term { const double* x; const double* y; double s; int order; int kind; };
  // kind 0: geta2phiz term, 1: phiz2 term, 2: phiz2 term whose gradeta2
  // product also enters geta2phiz2 at order + 2
  std::vector<Term> terms;
  for (int j = 1; j <= M - 3; ++j) terms.push_back({d.gradeta2, d.phizm[j], 1.0, j + 2, 0});
  if (M >= 3) terms.push_back({d.gradeta2, d.phizm[std::max(M - 2, 1)], 1.0, M, 0});
  for (int j = 1; j <= (M - 2) / 2; ++j) terms.push_back({d.phizm[j], d.phizm[j], 1.0, 2 * j, 2});
  for (int j = 2; j <= M - 3; ++j)
    for (int q = 1; q <= std::min(M - 2 - j, j - 1); ++q)
      terms.push_back({d.phizm[j], d.phizm[q], 2.0, j + q, 2});
  if (M >= 2) terms.push_back({d.phizm[M / 2], d.phizm[M / 2], 1.0, 2 * (M / 2), 1});
  for (int j = 2; j <= M - 1; ++j)
    for (int q = std::max(0, std::min(M - 2 - j, j - 1)) + 1; q <= std::min(M - j, j - 1); ++q)
      terms.push_back({d.phizm[j], d.phizm[q], 2.0, j + q, 1});
  auto cls = [&](int order) { return (E.act_x(order) ? 1 : 0) | (E.act_y(order) ? 2 : 0); };
  // groups keyed by (kind, class(order), class(order+2) for kind 2)
  std::vector<int> gkind, gc1, gc2;
  GroupTerms gt{};
  gt.nterm = 0;
  for (const Term& t : terms) {
    const int c1 = cls(t.order), c2 = t.kind == 2 ? cls(t.order + 2) : 0;
    int g = -1;
    for (size_t q = 0; q < gkind.size(); ++q)
      if (gkind[q] == t.kind && gc1[q] == c1 && gc2[q] == c2) g = (int)q;
    if (g < 0) {
      g = (int)gkind.size();
      gkind.push_back(t.kind);
      gc1.push_back(c1);
      gc2.push_back(c2);
    }
    gt.x[gt.nterm] = t.x;
    gt.y[gt.nterm] = t.y;
    gt.s[gt.nterm] = t.s;
    gt.group[gt.nterm] = g;
    gt.nterm++;
  }
  gt.ngroup = (int)gkind.size();
  for (int g = 0; g < gt.ngroup; ++g) gt.out[g] = d.grp[g];
  AssembleArgs aa{};
  aa.ng1 = aa.ng2 = aa.nt1 = 0;
  // fields dealiased together after the products
  std::vector<std::pair<int, double*>> dl = dl_late;
  for (int q = 0; q < 16; ++q) gt.outer_of[q] = -1;
  gt.nouter = 0;
  gt.oscale = d.gradeta2;
  if (gt.ngroup > 0) {
    // geta2phiz2: gradeta2 times the kind-2 groups, dealiased by outer class.
    // When no kind-2 group is dealiased itself, the products kernel forms
    // these sums too and everything is dealiased in one batch.
    bool fused = true;
    for (int g = 0; g < gt.ngroup; ++g)
      if (gkind[g] == 2 && gc1[g] != 0) fused = false;
    if (fused) {
      for (int c2 = 0; c2 < 4; ++c2) {
        bool any = false;
        for (int g = 0; g < gt.ngroup; ++g)
          if (gkind[g] == 2 && gc2[g] == c2) {
            gt.outer_of[g] = gt.nouter;
            any = true;
          }
        if (!any) continue;
        double* o = d.grp[gt.ngroup + gt.nouter];
        gt.out_outer[gt.nouter++] = o;
        dl.push_back({c2, o});
        aa.g2[aa.ng2++] = o;
      }
      E.ew(k_group_products, nB, gt, nB);
      for (int g = 0; g < gt.ngroup; ++g) dl.push_back({gc1[g], d.grp[g]});
    } else {
      E.ew(k_group_products, nB, gt, nB);
      {
        std::vector<std::pair<int, double*>> dl1;
        for (int g = 0; g < gt.ngroup; ++g) dl1.push_back({gc1[g], d.grp[g]});
        E.dealias_many(dl1);
      }
      int nu_ = 0;
      for (int c2 = 0; c2 < 4; ++c2) {
        SumArgs sa{};
        sa.nin = 0;
        for (int g = 0; g < gt.ngroup; ++g)
          if (gkind[g] == 2 && gc2[g] == c2) sa.in[sa.nin++] = d.grp[g];
        if (sa.nin == 0) continue;
        sa.scale = d.gradeta2;
        sa.out = d.grp[gt.ngroup + nu_];
        E.ew(k_sum_fields, nB, sa, nB);
        dl.push_back({c2, sa.out});
        aa.g2[aa.ng2++] = sa.out;
        nu_++;
      }
    }
    for (int g = 0; g < gt.ngroup; ++g) {
      if (gkind[g] == 0) aa.g1[aa.ng1++] = d.grp[g];
      else aa.t1[aa.nt1++] = d.grp[g];
    }
  }

  // 7. free-surface terms, filters to the n grid, final RHS
  aa.etax = d.etax; aa.etay = d.etay; aa.phisx = d.phisx; aa.phisy = d.phisy;
  aa.pxe = d.pxe; aa.pye = d.pye; aa.pze = d.pze;
  aa.detext = aa.dphext = nullptr;
  if (E.dealias_on(2)) {
    E.ew(k_fs_products, nB, (const double*)d.etax, (const double*)d.etay, (const double*)d.phisx,
         (const double*)d.phisy, d.tbig, d.tbig2, nB);
    dl.push_back({E.dclass(2), d.tbig});
    dl.push_back({E.dclass(2), d.tbig2});
    aa.detext = d.tbig;
    aa.dphext = d.tbig2;
  }
  E.dealias_many(dl);
  aa.nphizm = 0;
  for (int j = 1; j <= M - 1; ++j) aa.phizm[aa.nphizm++] = d.phizm[j];
  aa.phizmM = d.phizm[M];
  aa.M = M;
  cudaStreamWaitEvent(st, c.ev_join, 0);
  E.ew(k_assemble, nB, aa, d.A1, d.A3, nB);
  // filter_ext: S2F_big truncated to n1 x n2, then F2S on the n grid
  E.xf({E.R(GRID_BIG, 1, 0, 0, d.A1, nd1, nd1, nd2, d.pmode[0], n1, n1, n2),
        E.R(GRID_BIG, 1, 0, 0, d.phizm[1], nd1, nd1, nd2, d.pmode[1], n1, n1, n2),
        E.R(GRID_BIG, 1, 0, 0, d.A3, nd1, nd1, nd2, d.pmode[2], n1, n1, n2)});
  E.xf({E.F2S_N(d.pmode[0], d.X1), E.F2S_N(d.pmode[1], d.X2), E.F2S_N(d.pmode[2], d.X3)});
  E.ew(k_final, nN, (const double*)d.X1, (const double*)d.X2, (const double*)d.X3,
       (const double*)d.phiz_add, (const double*)d.phit_add, (const double*)d.nu, d.det, d.dph, nN,
       M);
  E.xf({E.S2F_N(d.det, d.NL1), E.S2F_N(d.dph, d.NL2)});
  E.ew_trig(k_expon, nN, (const double*)d.NL1, (const double*)d.NL2, (const double*)d.omega,
       (const double*)d.sc, kG1, kG2, nN, rk_mode ? 1 : 0);
}

void enqueue_step(Ctx& c, cudaStream_t st) {
  Enq E(c, st);
  const Params& P = c.P;
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const long long S = L.size;
  const long long nN = E.nN();
  // G1 = S2F(eta), G2 = S2F(phis) * omega
  E.xf({E.S2F_N(d.eta, d.y0 + L.off[S_G1]), E.S2F_N(d.phis, d.y0 + L.off[S_G2])});
  E.ew(k_scale_omega, nN, d.y0 + L.off[S_G2], (const double*)d.omega, d.sc, nN);
  // stage 1 at t_o
  {
    StageArgs sa{};
    sa.nk = 0;
    sa.c = 0.0;
    launch_pdl(k_rk_stage, dim3(nblk(S)), dim3(kEW), 0, st, d.y0, sa, d.sc, d.ys, S);
  }
  enqueue_rhs(c, d.ys, d.k[0], true, st);
  static const double A[5][5] = {{0, 0, 0, 0, 0}, {0.5, 0, 0, 0, 0}, {0, 0.5, 0, 0, 0},
                                 {0, 0, 1.0, 0, 0}, {-1.0, 2.0, 0, 0, 0}};
  static const double Cc[5] = {0.0, 0.5, 0.5, 1.0, 1.0};
  for (int s = 1; s < 5; ++s) {
    StageArgs sa{};
    sa.nk = 0;
    for (int j = 0; j < s; ++j) {
      sa.k[sa.nk] = d.k[j];
      sa.a[sa.nk] = A[s][j];
      sa.nk++;
    }
    sa.c = Cc[s];
    launch_pdl(k_rk_stage, dim3(nblk(S)), dim3(kEW), 0, st, d.y0, sa, d.sc, d.ys, S);
    enqueue_rhs(c, d.ys, d.k[s], true, st);
  }
  FinalArgs fa{};
  for (int j = 0; j < 5; ++j) fa.k[j] = d.k[j];
  for (int a = 0; a < 10; ++a) fa.off[a] = L.off[a];
  fa.off[10] = S;
  const int nb = nblk(S);
  launch_pdl(k_rk_final, dim3(nb), dim3(kEW), 0, st, d.y0, fa, d.sc, d.ynew, d.part, S);
  launch_pdl(k_rk_err, dim3(1), dim3(32), 0, st, d.part, nb, d.sc);
  launch_pdl(k_rk_out, dim3(nblk(nN, kTrig)), dim3(kTrig), 0, st, d.ynew + L.off[S_G1], d.ynew + L.off[S_G2],
                                     d.k[4] + L.off[S_G1], d.k[4] + L.off[S_G2], d.omega, d.sc,
                                     (int)nN, P.igeom, P.d_hinge, P.xlen, d.etam, d.phim, d.NL1,
                                     d.part + 10 * (long long)nb, d.counter);
  E.xf({E.F2S_N(d.etam, d.eta_c), E.F2S_N(d.phim, d.phis_c), E.F2S_N(d.NL1, d.deta_c)});
}

// ---------------------------------------------------------------------------
// Step control on the device (HOS-NWT.f90:498-571, as advance() in host.cpp)
// ---------------------------------------------------------------------------
// h_loc = h_rk, cut to reach time_next (HOS-NWT.f90:500-504); the step
// reads t_o and h_loc from the scalar slots
__global__ void k_ctl_begin(const StepCtl* __restrict__ ctl, double* __restrict__ sc) {
  pdl_wait();
  if (threadIdx.x == 0) {
    const double rem = ctl->time_next - ctl->time_cur;
    sc[SC_T0] = ctl->time_cur;
    sc[SC_H] = (rem < ctl->h_rk) ? rem : ctl->h_rk;
  }
}

// Accept / reject, dt_correc with the reference's REAL(4) constants, the
// clamps and the end of the ramp (HOS-NWT.f90:522-563); sets the loop
// condition: continue while time_cur < time_next.
__global__ void k_ctl_end(StepCtl* __restrict__ ctl, const double* __restrict__ sc, CtlParams p) {
  pdl_wait();
  if (threadIdx.x != 0) return;
  const double tiny = 2.220446049250313080847263336181640625e-16;  // epsilon(1.0_rp)
  const double error = sc[SC_ERR];
  const double h_loc = sc[SC_H];
  const double t = ctl->time_cur;
  double h_rk = ctl->h_rk;
  ctl->err = error;
  ctl->iters += 1;
  ctl->accept = 0;
  ctl->end_ramp_now = 0;
  if (!isfinite(error)) {
    ctl->status = 1;
    cudaGraphSetConditional(p.cond, 0);
    return;
  }
  double dt_correc;
  if (error > p.toler && h_rk > 0.001 * 0.95 * p.dt_stab) {
    dt_correc = (double)0.9f * pow(error / p.toler, -(double)(1.0f / 4.0f));
    ctl->n_rej += 1;
    if (fabs(p.Tramp - (t + h_loc)) <= tiny && p.Tramp > t) ctl->endramp = 0;
  } else {
    if (p.iramp == 1 && p.Tramp - (t + h_loc) <= tiny && p.Tramp > t && ctl->endramp != 1) {
      ctl->end_ramp_now = 1;
      ctl->endramp = 1;
    }
    ctl->accept = 1;
    ctl->time_cur = t + h_loc;
    dt_correc = fabs(error) < tiny ? 2.0 : 0.9 * pow(error / p.toler, -(1.0 / 4.0));
    ctl->n_acc += 1;
  }
  h_rk = h_rk * dt_correc;
  h_rk = fmin(fmin(h_rk, 0.95 * p.dt_stab), p.delt_out);
  h_rk = fmax(fmax(h_rk, 0.0001 * 0.95 * p.dt_stab), 0.0001 * p.delt_out);
  ctl->h_rk = h_rk;
  int go = ctl->time_cur < ctl->time_next ? 1 : 0;
  if (go && ctl->iters >= p.max_iters) {
    ctl->status = 2;
    go = 0;
  }
  cudaGraphSetConditional(p.cond, go);
}

// The accept of enqueue_accept, predicated on the decision: y0 <- ynew
// (less a_add_ramp in a_add_1 at the end of the ramp, HOS-NWT.f90:546-550),
// eta, phis, deta <- their candidates.
__global__ void k_accept_ctl(const StepCtl* __restrict__ ctl, double* __restrict__ y0,
                             const double* __restrict__ ynew, long long S, long long off1, long long offr,
                             long long nA, double* __restrict__ eta, const double* __restrict__ eta_c,
                             long long n2N, double* __restrict__ deta, const double* __restrict__ deta_c,
                             long long nN) {
  pdl_wait();
  if (!ctl->accept) return;
  const bool ramp = ctl->end_ramp_now != 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < S + n2N + nN; i += stride) {
    if (i < S) {
      double v = ynew[i];
      if (ramp && i >= off1 && i < off1 + nA) v -= ynew[offr + (i - off1)];
      y0[i] = v;
    } else if (i < S + n2N) {
      eta[i - S] = eta_c[i - S];
    } else {
      deta[i - S - n2N] = deta_c[i - S - n2N];
    }
  }
}

void enqueue_ctl_step(Ctx& c, StepCtl* ctl, const CtlParams& p, cudaStream_t st) {
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const long long nN = (long long)c.P.n1 * c.P.n2;
  const long long nA = (long long)c.P.n3a * c.P.n2;
  launch_pdl(k_ctl_begin, dim3(1), dim3(32), 0, st, (const StepCtl*)ctl, d.sc);
  enqueue_step(c, st);
  launch_pdl(k_ctl_end, dim3(1), dim3(32), 0, st, ctl, (const double*)d.sc, p);
  const long long tot = L.size + 3 * nN;
  const int blocks = (int)std::min<long long>((tot + kEW - 1) / kEW, 4LL * 152);
  launch_pdl(k_accept_ctl, dim3(blocks), dim3(kEW), 0, st, (const StepCtl*)ctl, d.y0, (const double*)d.ynew,
             L.size, L.off[S_AADD1], L.off[S_AADDR], nA, d.eta, (const double*)d.eta_c, 2 * nN, d.deta,
             (const double*)d.deta_c, nN);
}

void enqueue_accept(Ctx& c, bool end_ramp, cudaStream_t st) {
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  const long long nN = (long long)c.P.n1 * c.P.n2;
  cudaMemcpyAsync(d.y0, d.ynew, sizeof(double) * L.size, cudaMemcpyDeviceToDevice, st);
  // eta, phis are adjacent, and so are eta_c, phis_c
  cudaMemcpyAsync(d.eta, d.eta_c, sizeof(double) * 2 * nN, cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(d.deta, d.deta_c, sizeof(double) * nN, cudaMemcpyDeviceToDevice, st);
  if (end_ramp) {
    const long long nA = (long long)c.P.n3a * c.P.n2;
    launch_pdl(k_sub, dim3(nblk(nA)), dim3(kEW), 0, st, d.y0 + L.off[S_AADD1], d.y0 + L.off[S_AADDR], nA);
  }
}

// initialize (initial_condition.f90:314-482), wavemaker part: a1st_add from
// the initial paddle velocity, a_add_ramp = a1st_add, ramp/pos at t = 0.
void enqueue_initialize(Ctx& c, cudaStream_t st) {
  const Params& P = c.P;
  const Dev& d = c.d;
  const StateLayout& L = c.L;
  Enq E(c, st);
  cudaMemsetAsync(d.y0, 0, sizeof(double) * L.size, st);
  cudaMemsetAsync(d.deta, 0, sizeof(double) * E.nN(), st);
  enqueue_set_scalar(c, SC_TIME, 0.0, st);
  enqueue_set_scalar(c, SC_ALPHA, 0.0, st);
  enqueue_set_scalar(c, SC_ALPHAT, 0.0, st);
  enqueue_set_scalar(c, SC_ALPHATT, 0.0, st);
  enqueue_set_scalar(c, SC_POSTOP, 0.0, st);
  if (!has_wavemaker(P)) return;
  const RampP rp = ramp_params(P);
  const long long nA = E.nA();
  launch_pdl(k_eiwt, dim3(nblk(c.nf > 0 ? c.nf : 1)), dim3(kEW), 0, st, d.freq_w, d.sc, d.eiwt, c.nf, rp);
  launch_pdl(k_pos_bc, dim3(P.n2), dim3(128), 0, st, d.pos_re, d.pos_im, d.freq_w, d.eiwt, d.gzed, d.sc, c.nf,
                                 P.n2, P.n3, P.n3a, d.bc1, d.bcr, 1);
  {
    const int tot = (P.n3a - P.n3) * P.n2;
    launch_pdl(k_extend, dim3(nblk(tot)), dim3(kEW), 0, st, d.bc1, nullptr, d.ext, P.n2, P.n3, P.n3a);
  }
  double* a1 = d.y0 + L.off[S_AADD1];
  E.xf({E.R(GRID_ADD, 1, 0, 0, d.bc1, P.n3a, P.n3a, P.n2, a1, P.n3a, P.n3a, P.n2)});
  E.ew(k_div, nA, a1, (double*)nullptr, (const double*)d.k_add_thk, nA);
  cudaMemcpyAsync(d.y0 + L.off[S_AADDR], a1, sizeof(double) * nA, cudaMemcpyDeviceToDevice, st);
}

void enqueue_diagnostics(Ctx& c, double* out, cudaStream_t st) {
  const Params& P = c.P;
  launch_pdl(k_diagnostics, dim3(1), dim3(1024), 0, st, c.d.eta, c.d.phis, c.d.phi_add, c.d.deta, c.d.etax, c.d.etay, P.n1, P.n2,
                                     (long long)P.nd1 * P.nd2, out);
}

// filtering_x / filtering_y with coeff_cut = 0.7 of phis and eta (check_slope)
void enqueue_slope_filter(Ctx& c, int dir, cudaStream_t st) {
  Enq E(c, st);
  const Params& P = c.P;
  const int nf = dir == 0 ? std::abs((int)(P.n1 * 0.7)) : std::abs((int)(P.n2 * 0.7));
  for (double* f : {c.d.phis, c.d.eta}) {
    E.xf({E.S2F_N(f, c.d.NL1)});
    launch_pdl(k_cut_modes, dim3(nblk(E.nN())), dim3(kEW), 0, st, c.d.NL1, P.n1, P.n2, nf, dir);
    E.xf({E.F2S_N(c.d.NL1, f)});
  }
}

void enqueue_probes(Ctx& c, cudaStream_t st) {
  if (c.nprobes <= 0) return;
  Enq E(c, st);
  E.xf({E.S2F_N(c.d.eta, c.d.NL2)});
  launch_pdl(k_probe_dot, dim3(c.nprobes), dim3(256), 0, st, c.d.NL2, c.d.mat_coscos, E.nN(), c.d.probe_out);
}

}  // namespace hos
