// Host driver of the GB300 HOS wave tank: input parsing, set-up (the
// reference's initiate_parameters, nondimensionalisation, time-step choice,
// meshes, wave synthesis, absorbing zone, spectral tables), the adaptive
// time loop, probe output and the C ABI (include/hosnwt.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tank.h"

namespace hos {

static const double PI = 3.141592653589793238462643383279502888419;
static const double TWOPI = 6.283185307179586476925286766559005768394;
static const double G = 9.81;
static const double TINY = 2.220446049250313080847263336181640625e-16;  // epsilon(1.0_rp)

static int fail(Ctx& c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  c.err = buf;
  return code;
}

// ---------------------------------------------------------------------------
// linear wave theory (linear_wave.f90)
// ---------------------------------------------------------------------------
static double xthx(double x) { return x * std::tanh(x); }

// dichoto (linear_wave.f90:427-466): same bisection and stopping rule
static double dichoto(double (*f)(double), double f0, double a, double b, double prec) {
  const double fa = f(a) - f0;
  if (fa * (f(b) - f0) >= 0.0) {
    if (std::fabs(f(a) - f0) < TINY) return a;
    if (std::fabs(f(b) - f0) < TINY) return b;
  }
  double x1 = a, x2 = b, x3 = 0.0;
  while (std::fabs(x1 - x2) > prec * std::fabs(x2)) {
    x3 = (x1 + x2) / 2.0;
    const double f3 = f(x3) - f0;
    if (std::fabs(f3) < TINY) return x3;
    if (fa * f3 < 0.0) x2 = x3;
    else x1 = x3;
  }
  return x3;
}

// wave_number_adim_r (linear_wave.f90:137-151)
static double wave_number_adim(double f, double prec) {
  const double w2 = (TWOPI * f) * (TWOPI * f);
  if (w2 < std::log(1.7976931348623157e308) - 1.0) return dichoto(xthx, w2, 0.0, 1.0e6, prec);
  return w2;
}

// wave_number_r (linear_wave.f90:119-133): dimensional depth h
static double wave_number_r(double f, double h, double prec) {
  const double w2h = (TWOPI * f) * (TWOPI * f) / G * h;
  if (w2h < std::log(1.7976931348623157e308) - 1.0) return dichoto(xthx, w2h, 0.0, 10000000.0, prec) / h;
  return (TWOPI * f) * (TWOPI * f) / G;
}

// TF_adim_new (linear_wave.f90:277-334), hinged and piston branches
static std::complex<double> transfer_function(const std::string& typ, double k, double hinge) {
  const std::complex<double> I(0.0, 1.0);
  std::complex<double> resu;
  if (typ == "hinged" || typ == "monofl") {
    const double d = hinge;
    if (k < 50 && k * d < 50) {
      resu = -I * k * (1.0 - d) * (2.0 * k + std::sinh(2.0 * k)) / (4.0 * std::sinh(k));
      resu = resu / (k * (1.0 - d) * std::sinh(k) + std::cosh(k * d) - std::cosh(k));
    } else if (k >= 50 && k * d < 50) {
      resu = -I * k * (1.0 - d) / (2.0 * k * (1.0 - d) - 2.0 + 4.0 * std::cosh(k * d) * std::exp(-k));
    } else if (k * (1.0 - d) >= 20) {
      resu = -I * 0.5;
    } else {
      resu = -I * k * (1.0 - d) / (2.0 * k * (1.0 - d) - 2.0 + 2.0 * std::exp(k * (d - 1.0)));
    }
  } else if (typ == "piston") {
    if (k < 50.0) resu = std::complex<double>(0.0, -(2.0 * k + std::sinh(2.0 * k)) / (4.0 * std::sinh(k) * std::sinh(k)));
    else resu = std::complex<double>(0.0, -0.5);
  } else {
    resu = 1.0;
  }
  return resu;
}

// SRAND/RAND of libgfortran (initial_condition.f90:246,253): the Park-Miller
// minimal standard generator, its value masked to 24 significant bits and
// returned as REAL(4).
struct GfortranRand {
  unsigned long long seed;
  explicit GfortranRand(int s) : seed(s ? (unsigned long long)s : 123459876ull) {}
  float next() {
    seed = (16807ull * seed) % 2147483647ull;
    const unsigned int v = (unsigned int)(seed - 1) & ~511u;
    return (float)v / (float)2147483646u;
  }
};

// ---------------------------------------------------------------------------
// match_surface_wmk (resol_wmkr.f90:1655-1741): polynomial coefficients for
// l_add = 2 (x_med = 1), alpha_add = 6, beta_add = 1/3.  They are linear in
// (f, df, d2f); the same expressions as the reference.
// ---------------------------------------------------------------------------
static void match_coeffs(double f, double df, double d2f, double c[4]) {
  const double x = 1.0, a = 6.0, b = 1.0 / 3.0;
  const double E = std::exp(-a * b);
  auto p = [](double v, int n) { double r = 1.0; for (int i = 0; i < n; ++i) r *= v; return r; };
  const double inv_det = 1.0 / (-320 * p(x, 13) * E * p(b, 4) + 128 * p(x, 13) * E * p(b, 3) +
                                288 * p(x, 13) * E * p(b, 5) - 112 * p(x, 13) * E * p(b, 6) +
                                16 * p(x, 13) * E * p(b, 7));
  const double x2 = x * x;
  c[0] = inv_det * (2 * (3 * x * p(b, 4) * df + 2 * x2 * p(b, 4) * df * a + f * a * a * x2 * p(b, 4) +
         3 * f * a * x * p(b, 4) + x2 * p(b, 4) * d2f + 3 * f * p(b, 4) - 12 * x * p(b, 3) * df -
         8 * x2 * p(b, 3) * df * a - 4 * f * a * a * x2 * p(b, 3) - 12 * f * a * x * p(b, 3) -
         4 * x2 * p(b, 3) * d2f - 12 * f * p(b, 3) + 4 * x2 * b * b * d2f + 8 * x2 * b * b * df * a +
         8 * f * b * b + 8 * f * a * x * b * b + 4 * f * a * a * x2 * b * b + 8 * x * b * b * df +
         8 * f * b + 8 * x * b * df + 8 * f * a * x * b + 8 * f) * (-1 + b) * p(x, 6) * E);
  c[1] = inv_det * (-2 * (24 * f - 20 * f * a * a * x2 * p(b, 3) + 24 * f * a * x * b +
         12 * x2 * b * b * d2f - 6 * f * a * a * x2 * p(b, 5) + 3 * f * x * p(b, 6) * a +
         f * x2 * p(b, 6) * a * a - 60 * f * a * x * p(b, 3) + 12 * f * a * a * x2 * b * b +
         15 * f * a * a * x2 * p(b, 4) + 45 * f * a * x * p(b, 4) - 18 * f * a * x * p(b, 5) +
         2 * x2 * p(b, 6) * df * a - 12 * x2 * p(b, 5) * df * a + 30 * x2 * p(b, 4) * df * a -
         40 * x2 * p(b, 3) * df * a + 24 * x2 * b * b * df * a + 24 * f * b * b - 60 * f * p(b, 3) +
         24 * f * b + 45 * f * p(b, 4) - 18 * f * p(b, 5) + 3 * f * p(b, 6) + 24 * f * a * x * b * b +
         3 * x * p(b, 6) * df - 18 * x * p(b, 5) * df + 45 * x * p(b, 4) * df - 60 * x * p(b, 3) * df +
         24 * x * b * b * df + x2 * p(b, 6) * d2f - 6 * x2 * p(b, 5) * d2f + 15 * x2 * p(b, 4) * d2f -
         20 * x2 * p(b, 3) * d2f + 24 * x * b * df) * (-1 + b) * p(x, 8) * E);
  c[2] = inv_det * (2 * (24 * f - 28 * f * a * a * x2 * p(b, 3) + 24 * f * a * x * b +
         12 * x2 * b * b * d2f - 12 * f * a * a * x2 * p(b, 5) + 10 * f * x * p(b, 6) * a +
         2 * f * x2 * p(b, 6) * a * a - 116 * f * a * x * p(b, 3) + 12 * f * a * a * x2 * b * b +
         27 * f * a * a * x2 * p(b, 4) + 129 * f * a * x * p(b, 4) - 60 * f * a * x * p(b, 5) +
         4 * x2 * p(b, 6) * df * a - 24 * x2 * p(b, 5) * df * a + 54 * x2 * p(b, 4) * df * a -
         56 * x2 * p(b, 3) * df * a + 24 * x2 * b * b * df * a + 24 * f * b * b - 116 * f * p(b, 3) +
         24 * f * b + 129 * f * p(b, 4) - 60 * f * p(b, 5) + 10 * f * p(b, 6) + 24 * f * a * x * b * b +
         10 * x * p(b, 6) * df - 60 * x * p(b, 5) * df + 129 * x * p(b, 4) * df - 116 * x * p(b, 3) * df +
         24 * x * b * b * df + 2 * x2 * p(b, 6) * d2f - 12 * x2 * p(b, 5) * d2f + 27 * x2 * p(b, 4) * d2f -
         28 * x2 * p(b, 3) * d2f + 24 * x * b * df) * (-1 + b) * p(x, 10) * E);
  c[3] = inv_det * (-2 * (8 * f - 12 * f * a * a * x2 * p(b, 3) + 8 * f * a * x * b +
         4 * x2 * b * b * d2f - 6 * f * a * a * x2 * p(b, 5) + 7 * f * x * p(b, 6) * a +
         f * x2 * p(b, 6) * a * a - 68 * f * a * x * p(b, 3) + 4 * f * a * a * x2 * b * b +
         13 * f * a * a * x2 * p(b, 4) + 87 * f * a * x * p(b, 4) - 42 * f * a * x * p(b, 5) +
         2 * x2 * p(b, 6) * df * a - 12 * x2 * p(b, 5) * df * a + 26 * x2 * p(b, 4) * df * a -
         24 * x2 * p(b, 3) * df * a + 8 * x2 * b * b * df * a + 8 * f * b * b - 132 * f * p(b, 3) +
         8 * f * b + 183 * f * p(b, 4) - 90 * f * p(b, 5) + 15 * f * p(b, 6) + 8 * f * a * x * b * b +
         7 * x * p(b, 6) * df - 42 * x * p(b, 5) * df + 87 * x * p(b, 4) * df - 68 * x * p(b, 3) * df +
         8 * x * b * b * df + x2 * p(b, 6) * d2f - 6 * x2 * p(b, 5) * d2f + 13 * x2 * p(b, 4) * d2f -
         12 * x2 * p(b, 3) * d2f + 8 * x * b * df) * (-1 + b) * p(x, 12) * E);
}

// Extension weights: row n3+r = sum_q E[r][q] * row(n3-4+q)
static std::vector<double> extension_matrix(int n3, int n3a, int l_add, double delz) {
  const int nrow = n3a - n3;
  std::vector<double> E((size_t)std::max(nrow, 0) * 4, 0.0);
  const double x_med = (double)l_add - 1.0, a = 6.0;
  for (int q = 0; q < 4; ++q) {
    double d[4] = {0, 0, 0, 0};
    d[q] = 1.0;  // rows n3-4, n3-3, n3-2, n3-1 (0-based)
    const double df = (d[1] - 4.0 * d[2] + 3.0 * d[3]) / (2.0 * delz);
    const double f = d[3];
    const double d2f = (-d[0] + 4.0 * d[1] - 5.0 * d[2] + 2.0 * d[3]) / (delz * delz);
    double c[4];
    match_coeffs(f, df, d2f, c);
    for (int r = 0; r < nrow; ++r) {
      const int i3 = n3 + r + 1;  // 1-based row
      const double xx = (double)(i3 - 1) / (double)(n3 - 1) - (double)l_add;
      const double xx2 = xx * xx;
      E[4 * r + q] = (((c[0] * xx2 + c[1]) * xx2 + c[2]) * xx2 + c[3]) * xx * std::exp(-a * (xx + x_med));
    }
  }
  return E;
}

// ---------------------------------------------------------------------------
// input_HOS-NWT.dat (input.f90:62-201)
// ---------------------------------------------------------------------------
static double parse_real(const std::string& s) {
  std::string t = s;
  for (char& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';
  return std::strtod(t.c_str(), nullptr);
}

static std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

}  // namespace hos

using namespace hos;

extern "C" int hosnwt_read_input(const char* path, hosnwt_input* out) {
  if (!path || !out) return HOSNWT_ERR_ARG;
  std::ifstream f(path);
  if (!f) return HOSNWT_ERR_IO;
  std::vector<std::string> lines;
  std::string ln;
  while (std::getline(f, ln)) lines.push_back(ln);
  std::memset(out, 0, sizeof(*out));
  // line layout: blank lines at 0,4,6,9,16,21,26,32,36,39,43
  int li = 0;
  auto val = [&](void) -> std::string {
    if (li >= (int)lines.size()) return std::string();
    const std::string& s = lines[li++];
    return s.size() > 52 ? s.substr(52) : std::string();
  };
  auto blank = [&]() { ++li; };
  auto R = [&](double& v) { v = parse_real(trim(val())); };
  auto I = [&](int& v) { v = (int)std::lround(parse_real(trim(val()))); };
  auto S = [&](char* dst) {
    std::string s = trim(val());
    std::strncpy(dst, s.c_str(), 255);
  };
  blank(); R(out->xlen); R(out->ylen); R(out->h);
  blank(); I(out->icase);
  blank(); I(out->islosh); R(out->aslosh);
  blank(); R(out->amp_mono); R(out->nu_mono); R(out->theta_mono); R(out->ph_mono); I(out->ibat); R(out->xd_mono);
  blank(); S(out->file_name); I(out->i_cut); R(out->nuc_low); R(out->nuc_high);
  blank(); R(out->Hs); R(out->Tp); R(out->gamma); I(out->iseed);
  blank(); I(out->i_wmk); I(out->igeom); R(out->d_hinge); I(out->iramp); R(out->Tramp);
  blank(); I(out->iabsnb); R(out->xabsf); R(out->coeffabsf);
  blank(); I(out->iprobes); S(out->pro_file);
  blank(); R(out->T_stop); R(out->toler); R(out->f_out);
  blank(); I(out->idim); I(out->i3d); I(out->imodes); I(out->iwmk); I(out->i_sw);
  if (li > (int)lines.size()) return HOSNWT_ERR_IO;
  return HOSNWT_OK;
}

namespace hos {

// ---------------------------------------------------------------------------
// set-up
// ---------------------------------------------------------------------------
static double gzed_fn(const Params& P, double z) {
  // gzed (wavemaking.f90:184-213)
  const double dh = P.d_hinge;
  const double delta = std::min(dh, (1.0 - dh) / 10.0);
  if (P.igeom == 1) return 1.0;
  if (z >= (dh - 1.0 + delta)) return (z + 1.0 - dh) / (1.0 - dh);
  if (z <= (dh - 1.0 - delta)) return 0.0;
  const double U = z - (dh - 1.0);
  const double u = U / delta;
  return delta / (2.0 * (1.0 - dh)) *
         (5.0 / 16.0 + u + 15.0 / 16.0 * (u * u - 1.0 / 3.0 * u * u * u * u + 1.0 / 15.0 * u * u * u * u * u * u));
}

static double dgzeddz_fn(const Params& P, double z) {
  // dgzeddz (wavemaking.f90:222-250)
  const double dh = P.d_hinge;
  const double delta = std::min(dh, (1.0 - dh) / 10.0);
  if (P.igeom == 1) return 0.0;
  if (z >= (dh - 1.0 + delta)) return 1.0 / (1.0 - dh);
  if (z <= (dh - 1.0 - delta)) return 0.0;
  const double u = (z - (dh - 1.0)) / delta;
  return 1.0 / (1.0 - dh) * (1.0 / 2.0 + 15.0 / 16.0 * (u - 2.0 / 3.0 * u * u * u + 1.0 / 5.0 * u * u * u * u * u));
}

struct Wave {
  std::vector<int> harmo;
  std::vector<double> freq, ampli, angle, phase, k;
  std::vector<std::complex<double>> TF;
  int rnum = 1;
  double clock = 0.0, depth = 0.0;
};

// phase (wave_def.f90:491-523) as the reference writes it: its first test
// returns 0 for every |z| > tiny, so only |z| <= tiny reaches the angle
// formula.  Results match the reference's Benchmark/Regular_3D output only
// with this behaviour.
static double fortran_phase(std::complex<double> z) {
  if (std::abs(z) > TINY) return 0.0;
  const std::complex<double> zt = z / std::abs(z);
  const double pt = std::asin(zt.imag());
  if (zt.real() >= 0.0) return zt.imag() >= 0.0 ? pt : TWOPI + pt;
  return PI - pt;
}

// dalrymple (wave_def.f90:111-177): an oblique wave of one frequency as
// 2 (N+1) components over the tank's y-modes, focused at x = X_d;
// appended to w (add_wave, wave_def.f90:333-384).
static void dalrymple_append(Wave& w, double Ly, double X_d, int harmo, double ampli, double angle,
                             double phas) {
  using cd = std::complex<double>;
  const cd I(0.0, 1.0);
  const double freq = harmo * w.clock / std::pow(2.0, w.rnum);
  const double k = wave_number_adim(freq, 1.0e-12);
  const int N = (int)std::floor(k * Ly / PI);
  const double beta = k * std::sin(angle);
  std::vector<cd> a_on(N + 1);
  std::vector<double> theta(N + 1);
  cd tmp = -std::exp(-I * beta * Ly);
  for (int n = 0; n <= N; ++n) {
    const double mu = n * PI / Ly;
    theta[n] = std::asin(mu / k);
    const double delta = n == 0 ? 1.0 : 0.0;
    cd In;
    if (std::fabs(angle) < TINY) {
      In = delta;
    } else {
      tmp = -tmp;
      if (std::fabs(mu - std::fabs(beta)) < TINY) In = 1.0;
      else In = 2.0 * I * beta * (tmp - 1.0) / (beta * beta - mu * mu) / ((1.0 + delta) * Ly);
    }
    const cd kn = I * std::sqrt(k * k - mu * mu);
    a_on[n] = ampli * std::exp(I * phas) * In * std::exp((kn - I * k * std::cos(angle)) * X_d);
  }
  for (int half = 0; half < 2; ++half)
    for (int n = 0; n <= N; ++n) {
      w.harmo.push_back(harmo);
      w.freq.push_back(freq);
      w.ampli.push_back(std::abs(a_on[n] / 2.0));
      w.angle.push_back(half == 0 ? theta[n] : -theta[n]);
      w.phase.push_back(fortran_phase(a_on[n]));
    }
}

static void wave_init(Wave& w, const std::string& typ, double hinge) {
  // wave_init (wave_def.f90:282-329)
  const size_t n = w.freq.size();
  w.k.assign(n, 0.0);
  w.TF.assign(n, std::complex<double>(1.0, 0.0));
  for (size_t i = 0; i < n; ++i) {
    const double kt = wave_number_adim(w.freq[i], 1.0e-15);
    w.k[i] = kt;
    w.TF[i] = std::fabs(kt) > TINY ? transfer_function(typ, kt, hinge) : std::complex<double>(1.0, 0.0);
    if (w.freq[i] < 1.0e-8) {
      w.k[i] = 0.0;
      w.TF[i] = 1.0;
    }
  }
}

// ocean_txt2cfg_dat (read_ocean_txt.f90:33-228) for the ECN wave basin
// (icase 31) and towing tank (32): the fronts of an Edinburgh Designs .txt
// file as the lines of the .cfg and .dat files the reference writes and then
// reads back (the .dat values pass through G20.7, 7 significant digits).
static int ocean_txt2cfg_dat(const std::string& path, int i_cut, double nuc_low, double nuc_high, int icase,
                             std::vector<std::string>& cfg, std::vector<std::string>& dat) {
  std::ifstream f(path);
  if (!f) return 1;
  std::vector<std::string> lines;
  std::string t;
  while (std::getline(f, t)) lines.push_back(t);
  int rnum = -1, ramp = 0, rcomp = 0, n_front = -1;
  size_t n_start = 0;
  auto after = [](const std::string& s, const std::string& key) {
    std::istringstream is(s.substr(s.find(key) + key.size()));
    long long v = 0;
    is >> v;
    return v;
  };
  for (size_t i = 0; i < lines.size(); ++i) {
    const std::string& s = lines[i];
    if (s.find("rnumber  =") != std::string::npos) rnum = (int)after(s, "=");
    if (s.find("ramp     =") != std::string::npos) ramp = (int)after(s, "=");
    if (s.find("rnumber compression") != std::string::npos) rcomp = (int)after(s, s.substr(0, s.rfind('=') + 1));
    if (s.find("Wave has ") != std::string::npos) {
      n_front = (int)after(s, "Wave has ");
      n_start = i + 2;
    }
  }
  if (rnum < 0 || n_front < 0 || n_start + n_front > lines.size()) return 1;
  const double clock = 32.0, f_base = clock / std::pow(2.0, rnum);
  const double f_lo = i_cut == 1 ? nuc_low : 0.0, f_hi = i_cut == 1 ? nuc_high : 100.0;
  char buf[128];
  auto F = [&](const char* fmt, double v) { std::snprintf(buf, sizeof buf, fmt, v); return std::string(buf); };
  cfg = {F("%2.0f", rnum), F("%5.2f", clock), F("%5.2f", icase == 31 ? 5.0 : 2.88), F("%4.0f", ramp), "lin",
         F("%5.2f", f_lo), F("%6.2f", f_hi), F("%5.2f", icase == 31 ? 30.0 : 5.0), "hinged",
         F("%6.3f", icase == 31 ? 2.147 : 0.0)};
  dat.clear();
  auto g7 = [&](double v) { std::snprintf(buf, sizeof buf, "%.6E", v); return std::string(buf); };
  for (int j = 0; j < n_front; ++j) {
    std::istringstream is(lines[n_start + j]);
    double h, fr, a, ang, ph;
    is >> h >> fr >> a >> ang >> ph;
    long long harmo = std::llround(h);
    if (rcomp) harmo *= rcomp;
    const double freq = harmo * f_base;
    if (icase == 31) ph = ph + wave_number_r(freq, 5.0, 1.0e-12) * 29.74 / 2.0 * std::sin(ang);
    ang = 180.0 * ang / PI;
    if (a < 1.0e-98) a = 0.0;
    if (freq >= f_lo && freq <= f_hi)
      dat.push_back(std::to_string(harmo) + " " + g7(freq) + " " + g7(a) + " " + g7(ang) + " " + g7(ph));
  }
  return 0;
}

static int wave_cfg(Ctx& c, const char* wave_dir) {
  // initialize_wav_cfg (initial_condition.f90:128-310)
  Params& P = c.P;
  const hosnwt_input& in = c.in;
  std::string typ = P.igeom == 2 ? "hinged" : "piston";
  Wave w;
  double hinge = P.d_hinge;
  if (P.icase == 1) {
    c.nf = 0;
  } else if (P.icase == 2) {
    if (in.ibat != 2 && in.ibat != 3)
      return fail(c, HOSNWT_ERR_UNSUPPORTED, "only snake (ibat=2) and Dalrymple (ibat=3) wavemaking");
    w.rnum = 1;
    w.clock = 2.0 * P.nu_mono;
    w.depth = P.h;
    if (in.ibat == 3) {
      dalrymple_append(w, P.ylen, in.xd_mono / P.h, 1, P.amp_mono, P.theta_mono, P.ph_mono);
    } else {
      w.harmo = {1};
      w.freq = {1 * w.clock / (double)(1 << w.rnum)};
      w.ampli = {P.amp_mono};
      w.angle = {P.theta_mono};
      w.phase = {P.ph_mono};
    }
  } else if (P.icase == 3 || P.icase == 31 || P.icase == 32) {
    std::string base = std::string(wave_dir ? wave_dir : ".") + "/" + trim(in.file_name);
    std::vector<std::string> cl, dl;  // the .cfg and .dat lines
    std::string s;
    if (P.icase == 3) {
      std::ifstream cf(base + ".cfg");
      if (!cf) return fail(c, HOSNWT_ERR_IO, "cannot open %s.cfg", base.c_str());
      while (std::getline(cf, s)) cl.push_back(trim(s));
      std::ifstream df(base + ".dat");
      if (!df) return fail(c, HOSNWT_ERR_IO, "cannot open %s.dat", base.c_str());
      while (std::getline(df, s)) dl.push_back(s);
    } else {
      const int rc = ocean_txt2cfg_dat(base + ".txt", in.i_cut, in.nuc_low, in.nuc_high, P.icase, cl, dl);
      if (rc) return fail(c, HOSNWT_ERR_IO, "cannot read the ocean file %s.txt", base.c_str());
    }
    if (cl.size() < 10) return fail(c, HOSNWT_ERR_IO, "short .cfg file");
    auto first = [&](int i) { std::istringstream is(cl[i]); std::string t; is >> t; return t; };
    w.rnum = std::atoi(first(0).c_str());
    const double clock_d = parse_real(first(1));
    w.depth = parse_real(first(2));
    const double cut_lo = parse_real(first(5)), cut_hi = parse_real(first(6));
    typ = first(8);
    const double hinge_d = parse_real(first(9));
    const double Ts = std::sqrt(w.depth / G);
    w.clock = clock_d * Ts;
    const double cut_lo_n = cut_lo * Ts, cut_hi_n = cut_hi * Ts;
    hinge = hinge_d / w.depth;
    std::vector<int> ha;
    std::vector<double> fa, aa, ga, pa;
    for (std::string s : dl) {
      if (trim(s).empty()) continue;
      for (char& ch : s)
        if (ch == ',') ch = ' ';
      std::istringstream is(s);
      std::string t0, t1, t2, t3, t4;
      is >> t0 >> t1 >> t2 >> t3 >> t4;
      ha.push_back((int)std::lround(parse_real(t0)));
      fa.push_back(parse_real(t1));
      aa.push_back(parse_real(t2));
      ga.push_back(parse_real(t3));
      pa.push_back(parse_real(t4));
    }
    int n_start = 1, n_stop = 0;  // wave_def.f90:240-248
    for (size_t i = 0; i < fa.size(); ++i) {
      if (fa[i] <= cut_hi_n / Ts) n_stop = (int)i + 1;
      if (fa[i] < cut_lo_n / Ts) n_start++;
    }
    if (n_stop - n_start + 1 <= 0) return fail(c, HOSNWT_ERR_ARG, "n_good == 0");
    for (int i = n_start - 1; i < n_stop; ++i) {
      w.harmo.push_back(ha[i]);
      w.freq.push_back(fa[i] * Ts);
      w.ampli.push_back(aa[i] / w.depth);
      w.angle.push_back(ga[i] * PI / 180.0);
      w.phase.push_back(pa[i]);
    }
    if (in.ibat == 3 && P.n2 != 1) {
      // initial_condition.f90:192-199: the Dalrymple waves of every component
      Wave src = w;
      w.harmo.clear(); w.freq.clear(); w.ampli.clear(); w.angle.clear(); w.phase.clear();
      for (size_t i = 0; i < src.harmo.size(); ++i)
        dalrymple_append(w, P.ylen, in.xd_mono / P.h, src.harmo[i], src.ampli[i], src.angle[i], src.phase[i]);
    }
  } else if (P.icase == 4) {
    const double Tp = in.Tp, Hs = in.Hs, gam = in.gamma;
    const double clock = 32.0;
    w.rnum = (int)std::ceil(std::log10(P.T_stop * P.Tscale * clock) / std::log10(2.0));
    w.depth = P.h;
    const int n_pts = (int)std::lround(2 * std::pow(2.0, w.rnum) / clock + 1);
    const double f_base = (double)(float)clock / std::pow(2.0, w.rnum);
    GfortranRand rnd(in.iseed);
    double Hs_int = 0.0;
    const double sig_lo = (double)0.07f, sig_hi = (double)0.09f;
    for (int i1 = 1; i1 <= n_pts; ++i1) {
      const double fr = i1 * f_base;
      w.harmo.push_back(i1 - 1);
      w.freq.push_back(fr);
      w.angle.push_back(0.0);
      w.phase.push_back(TWOPI * (double)rnd.next());
      const double sigma = fr < 1.0 / Tp ? sig_lo : sig_hi;
      const double a = 1.0 / std::pow(TWOPI, 4) * G * G / std::pow(fr, 5) *
                       std::exp(-5.0 / 4.0 * std::pow(fr * Tp, -4)) *
                       std::pow(gam, std::exp((-(fr - 1.0 / Tp) * (fr - 1.0 / Tp)) / (2.0 * (sigma / Tp) * (sigma / Tp)))) * f_base;
      Hs_int += a;
      w.ampli.push_back(std::sqrt(2.0 * a));
    }
    Hs_int = 4.0 * std::sqrt(Hs_int);
    for (size_t i = 0; i < w.ampli.size(); ++i) {
      w.ampli[i] = w.ampli[i] * Hs / Hs_int / P.h;
      w.freq[i] = w.freq[i] * P.Tscale;
    }
    w.clock = clock * P.Tscale;
  } else {
    return fail(c, HOSNWT_ERR_UNSUPPORTED, "icase=%d is not supported", P.icase);
  }
  c.gzed.resize(P.n3);
  for (int i3 = 0; i3 < P.n3; ++i3) c.gzed[i3] = gzed_fn(P, c.cz[i3]);
  if (P.icase == 1) return HOSNWT_OK;
  wave_init(w, typ, hinge);
  if (!w.k.empty()) {
    c.k_mono = w.k[0];
    if (std::fabs(c.k_mono) < TINY && w.k.size() > 1) c.k_mono = w.k[1];
  }
  // wmk_ini (wavemaking.f90:37-175), full-width wavemaker
  int n_max = std::max(1, (int)std::floor(w.clock * std::sqrt(G / w.depth)));
  n_max = (1 << w.rnum) / n_max;
  std::vector<std::vector<int>> groups;
  for (int harm = 0; harm <= 4 * n_max; ++harm) {
    std::vector<int> idx;
    for (size_t i = 0; i < w.harmo.size(); ++i)
      if (w.harmo[i] == harm) idx.push_back((int)i);
    if (!idx.empty()) groups.push_back(idx);
  }
  c.nf = (int)groups.size();
  c.freq_w.resize(c.nf);
  c.pos_ini.assign((size_t)P.n2 * c.nf, std::complex<double>(0.0, 0.0));
  c.dposdy_ini.assign((size_t)P.n2 * c.nf, std::complex<double>(0.0, 0.0));
  const std::complex<double> I(0.0, 1.0);
  for (int g = 0; g < c.nf; ++g) {
    c.freq_w[g] = w.freq[groups[g][0]];
    for (int j1 = 0; j1 < P.n2; ++j1) {
      std::complex<double> acc(0.0, 0.0), dacc(0.0, 0.0);
      for (int i : groups[g]) {
        const double ang = w.angle[i];
        const std::complex<double> tmp = w.TF[i] * std::cos(ang) * w.ampli[i] *
                                         std::exp(I * (-w.k[i] * std::sin(ang) * c.cy[j1] + w.phase[i]));
        acc += 1.0 * tmp;
        // dposdy_ini with rampy = 1, drampy = 0 (full-width wavemaker)
        dacc += (0.0 - I * w.k[i] * std::sin(ang) * 1.0) * tmp;
      }
      c.pos_ini[j1 + (size_t)P.n2 * g] = acc;
      c.dposdy_ini[j1 + (size_t)P.n2 * g] = dacc;
    }
  }
  return HOSNWT_OK;
}

template <typename T>
static T* dalloc(Ctx& c, size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, n * sizeof(T));
  c.allocs.push_back(p);
  return (T*)p;
}

static double* upload(Ctx& c, const std::vector<double>& v) {
  double* p = dalloc<double>(c, v.size());
  if (p && !v.empty()) cudaMemcpy(p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
  return p;
}

int setup(Ctx& c, const char* wave_dir, const double* probes_xy, int nprobes) {
  Params& P = c.P;
  const hosnwt_input& in = c.in;
  const hosnwt_numerics& nm = c.num;
  // check_range (initial_condition.f90:584-605) and initiate_parameters
  auto in_range = [](int v) {
    static const int ok[] = {1, 2, 3, 4, 5, 7, 8, 9, 11, 14, 15, 17, 19, 23, 29};
    for (int o : ok)
      if (o == v) return true;
    return false;
  };
  if (!in_range(nm.mHOS) || !in_range(nm.p1) || !in_range(nm.p2))
    return fail(c, HOSNWT_ERR_ARG, "forbidden value of M, p1 or p2");
  if (nm.p1 > nm.mHOS || nm.p2 > nm.mHOS) return fail(c, HOSNWT_ERR_ARG, "p1/p2 higher than M");
  if (nm.n1 < 5 || nm.n2 < 1 || (nm.n2 > 1 && nm.n2 < 5) || nm.n3 < 5)
    return fail(c, HOSNWT_ERR_ARG, "grid too small (n1, n3 >= 5; n2 = 1 or >= 5)");
  if (nm.mHOS > 11) return fail(c, HOSNWT_ERR_ARG, "mHOS > 11 is not supported");
  if (nm.n3 > 257) return fail(c, HOSNWT_ERR_ARG, "n3 > 257 (n3_add is limited to 512)");
  P.n1 = nm.n1; P.n2 = nm.n2; P.n3 = nm.n3; P.M = nm.mHOS; P.p1 = nm.p1; P.p2 = nm.p2;
  P.l_add = 2;
  P.n3a = P.l_add * (P.n3 - 1);
  P.nd1 = ((P.p1 + 1) * P.n1) / 2;
  P.nd2 = ((P.p2 + 1) * P.n2) / 2;
  if (P.n2 == 1) P.nd2 = 1;
  P.icase = in.icase; P.igeom = in.igeom; P.iramp = in.iramp; P.iabsnb = in.iabsnb;
  P.i_wmk = in.i_wmk; P.ibat = in.ibat;
  if (P.icase != 1 && (P.i_wmk < 1 || P.i_wmk > 3))
    return fail(c, HOSNWT_ERR_UNSUPPORTED, "the wavemaker order i_wmk must be 1, 2 or 3");
  if (P.icase != 1 && P.igeom != 1 && P.igeom != 2)
    return fail(c, HOSNWT_ERR_UNSUPPORTED, "only flap/piston wavemakers (igeom 1, 2) are supported");
  // nondimensionalisation (HOS-NWT.f90:99-119)
  P.h = in.h;
  P.Tscale = 1.0 / std::sqrt(G / P.h);
  P.xlen = in.xlen / P.h;
  P.ylen = in.ylen / P.h;
  P.amp_mono = in.amp_mono / P.h;
  P.xlen_add = 2.0 * (double)P.l_add;
  P.d_hinge = in.d_hinge / P.h;
  P.aslosh = in.aslosh / P.h;
  P.Tramp = in.iramp == 0 ? 0.0 : in.Tramp / P.Tscale;
  P.T_stop = in.T_stop / P.Tscale;
  P.f_out = in.f_out * P.Tscale;
  P.nu_mono = in.nu_mono * P.Tscale;
  P.w_mono = P.nu_mono * TWOPI;
  P.T_mono = 1.0 / P.nu_mono;
  P.theta_mono = (P.n2 != 1 ? in.theta_mono : 0.0) * PI / 180.0;
  P.ph_mono = in.ph_mono;
  P.islosh = in.islosh + 1;
  P.toler = in.toler;
  // time-step choice (HOS-NWT.f90:130-217)
  double dtr[3];
  dtr[0] = std::sqrt(8 / (PI * PI)) * P.xlen / (double)(float)(P.n1 - 1);
  dtr[1] = P.n2 != 1 ? std::sqrt(8 / (PI * PI)) * P.ylen / (double)(float)(P.n2 - 1) : dtr[0] + 1.0;
  dtr[2] = P.igeom != 3 ? std::sqrt(8 / (PI * PI)) * (2.0 * (double)P.l_add) / (double)(float)(P.l_add * (P.n3 - 1))
                        : dtr[0] + 1.0;
  double dt_stab;
  if (P.igeom == 3 || P.icase == 1) dt_stab = P.n2 == 1 ? dtr[0] : std::min(dtr[0], dtr[1]);
  else if (P.n2 == 1) dt_stab = std::min(dtr[0], dtr[2]);
  else dt_stab = std::min(std::min(dtr[0], dtr[1]), dtr[2]);
  P.dt_stab = dt_stab;
  P.delt_out = 1.0 / P.f_out;
  P.delt = std::min(0.95 * dt_stab, P.delt_out);
  if (std::fabs(P.delt - P.delt_out) < TINY) return fail(c, HOSNWT_ERR_ARG, "DECREASE f_out");
  // meshes (HOS-NWT.f90:220-244)
  P.delx = P.xlen / (P.n1 - 1);
  P.delz = 1.0 / (P.n3 - 1);
  P.dely = P.n2 != 1 ? P.ylen / (P.n2 - 1) : 0.0;
  c.cx.resize(P.n1);
  c.cy.resize(P.n2);
  c.cz.resize(P.n3);
  for (int i = 0; i < P.n1; ++i) c.cx[i] = i * P.delx;
  for (int i = 0; i < P.n2; ++i) c.cy[i] = i * P.dely;
  for (int i = 0; i < P.n3; ++i) c.cz[i] = P.delz * i - 1.0;
  int rc = wave_cfg(c, wave_dir);
  if (rc) return rc;
  // spectral tables (HOS-NWT.f90:267-406)
  const int n1 = P.n1, n2 = P.n2, nd1 = P.nd1, nd2 = P.nd2, M = P.M, n3a = P.n3a;
  const double pixlen = PI / P.xlen, piylen = n2 != 1 ? PI / P.ylen : 0.0;
  c.kx.resize(n1);
  c.ky.resize(n2);
  for (int i = 0; i < n1; ++i) c.kx[i] = i * pixlen;
  for (int i = 0; i < n2; ++i) c.ky[i] = i * piylen;
  c.omega.resize((size_t)n1 * n2);
  std::vector<double> kth1((size_t)n1 * n2);
  for (int i2 = 0; i2 < n2; ++i2)
    for (int i1 = 0; i1 < n1; ++i1) {
      const double k = std::sqrt(c.kx[i1] * c.kx[i1] + c.ky[i2] * c.ky[i2]);
      c.omega[i1 + (size_t)n1 * i2] = std::sqrt(k * std::tanh(k));
      kth1[i1 + (size_t)n1 * i2] = k * std::tanh(k);
    }
  std::vector<double> kth_ext((size_t)nd1 * nd2 * M);
  for (int i2 = 0; i2 < nd2; ++i2)
    for (int i1 = 0; i1 < nd1; ++i1) {
      const double kk = std::sqrt((i1 * pixlen) * (i1 * pixlen) + (i2 * piylen) * (i2 * piylen));
      const double thk = std::tanh(kk);
      double pw = 1.0;
      for (int j = 1; j <= M; ++j) {
        pw = std::pow(kk, j);
        kth_ext[i1 + (size_t)nd1 * i2 + (size_t)nd1 * nd2 * (j - 1)] = (j % 2 == 1) ? pw * thk : pw;
      }
    }
  // wavemaker modes and the exponential tables with the 700 guard
  const double pixlen_add = PI / P.xlen_add;
  std::vector<double> kx_add(n3a), cosk(n3a), sink(n3a), k_add((size_t)n3a * n2), k_add_thk((size_t)n3a * n2);
  for (int i3 = 0; i3 < n3a; ++i3) {
    kx_add[i3] = (2 * (i3 + 1) - 1) * pixlen_add;
    cosk[i3] = std::cos(kx_add[i3]);
    sink[i3] = std::sin(kx_add[i3]);
    for (int i2 = 0; i2 < n2; ++i2) {
      const double ka = std::sqrt(kx_add[i3] * kx_add[i3] + c.ky[i2] * c.ky[i2]);
      k_add[i3 + (size_t)n3a * i2] = ka;
      k_add_thk[i3 + (size_t)n3a * i2] = ka * std::tanh(ka * P.xlen);
    }
  }
  const size_t nT = (size_t)n1 * n3a * n2;
  std::vector<double> csh(nT), ksh(nT), kycsh(nT), kxcsh(nT);
  const double XMAX = 700.0;
  for (int i2 = 0; i2 < n2; ++i2)
    for (int i3 = 0; i3 < n3a; ++i3) {
      const double ka = k_add[i3 + (size_t)n3a * i2], ka2 = 2.0 * ka;
      const double kxl = ka2 * P.xlen;
      const double e3 = kxl <= XMAX ? std::exp(-ka2 * P.xlen) : 0.0;
      const double e3p1 = e3 + 1.0;
      for (int i1 = 0; i1 < n1; ++i1) {
        const double x1 = ka * c.cx[i1];
        const double e1 = x1 <= XMAX ? std::exp(-x1) / e3p1 : 0.0;
        const double x2 = ka2 * (P.xlen - c.cx[i1]);
        const double e2 = x2 <= XMAX ? std::exp(-x2) : 0.0;
        const double e12 = (x1 + x2 <= XMAX) ? e1 * e2 : 0.0;
        const double ch = e1 + e12, sh = e1 - e12;
        const size_t o = i1 + (size_t)n1 * i3 + (size_t)n1 * n3a * i2;
        csh[o] = ch;
        ksh[o] = sh * ka;
        kycsh[o] = ch * c.ky[i2];
        kxcsh[o] = ch * kx_add[i3];
      }
    }
  // absorbing zone (initial_condition.f90:724-794), full width, front beach only
  std::vector<double> nu((size_t)n1 * n2, 0.0);
  if (P.iabsnb != 0) {
    const double x0 = P.xlen * in.xabsf;
    if (std::fabs(in.xabsf - 1.0) > TINY) {
      const double x2 = P.xlen - x0;
      for (int i1 = 0; i1 < n1; ++i1)
        if (c.cx[i1] >= x0) {
          const double x3 = (c.cx[i1] - x0) / x2;
          for (int i2 = 0; i2 < n2; ++i2) nu[i1 + (size_t)n1 * i2] = in.coeffabsf * x3 * x3;
        }
    }
  }
  // probes (initialize_probes_matrices, initial_condition.f90:496-501)
  c.nprobes = (probes_xy && nprobes > 0) ? nprobes : 0;
  std::vector<double> mat((size_t)n1 * n2 * std::max(c.nprobes, 1), 0.0);
  c.probes.assign(2 * (size_t)c.nprobes, 0.0);
  for (int p = 0; p < c.nprobes; ++p) {
    const double xp = probes_xy[2 * p] / P.h, yp = probes_xy[2 * p + 1] / P.h;
    c.probes[2 * p] = xp;
    c.probes[2 * p + 1] = yp;
    for (int i2 = 0; i2 < n2; ++i2)
      for (int i1 = 0; i1 < n1; ++i1)
        mat[i1 + (size_t)n1 * i2 + (size_t)n1 * n2 * p] = std::cos(c.kx[i1] * xp) * std::cos(c.ky[i2] * yp);
  }
  // state layout
  long long o = 0;
  const long long nN = (long long)n1 * n2, nA = (long long)n3a * n2;
  const long long sz[10] = {nN, nN, nA, nA, nA, nA, nN, nN, nN, nN};
  for (int a = 0; a < 10; ++a) { c.L.off[a] = o; o += sz[a]; }
  c.L.size = o;
  // device
  if (alloc_device(c)) return fail(c, HOSNWT_ERR_CUDA, "device allocation failed");
  Dev& d = c.d;
  d.omega = upload(c, c.omega);
  d.kx = upload(c, c.kx);
  d.ky = upload(c, c.ky);
  d.kth_ext = upload(c, kth_ext);
  d.kth1 = upload(c, kth1);
  d.nu = upload(c, nu);
  d.k_add_thk = upload(c, k_add_thk);
  d.kx_add = upload(c, kx_add);
  d.cosk = upload(c, cosk);
  d.sink = upload(c, sink);
  d.csh = upload(c, csh);
  d.ksh = upload(c, ksh);
  d.kycsh = upload(c, kycsh);
  d.kxcsh = upload(c, kxcsh);
  d.ext = upload(c, extension_matrix(P.n3, n3a, P.l_add, P.delz));
  if (P.i_wmk >= 2) {
    // second- and third-order wavemaker (d1st_for_2nd, SWEET_2, SWEET_3): free-surface
    // modes on the wavemaker (HOS-NWT.f90:343-355), [i1 + n1 (i2 + n2 i3)]
    const int n3 = P.n3;
    std::vector<double> kx2c((size_t)n1 * n2 * n3), kyc(kx2c.size()), ks(kx2c.size());
    for (int i3 = 0; i3 < n3; ++i3)
      for (int i2 = 0; i2 < n2; ++i2)
        for (int i1 = 0; i1 < n1; ++i1) {
          const double kk = std::sqrt(c.kx[i1] * c.kx[i1] + c.ky[i2] * c.ky[i2]);
          const double cxk = kk * (P.delz * i3), ch = std::cosh(kk);
          const double cshx = std::cosh(cxk) / ch;
          const size_t o = i1 + (size_t)n1 * (i2 + (size_t)n2 * i3);
          kx2c[o] = cshx * c.kx[i1] * c.kx[i1];
          kyc[o] = cshx * c.ky[i2];
          ks[o] = kk * std::sinh(cxk) / ch;
        }
    d.kx2cshx = upload(c, kx2c);
    d.kycshx = upload(c, kyc);
    d.kshx = upload(c, ks);
    d.k_add = upload(c, k_add);
    // dnux as absorb writes it: coeffabsf * 2 * x3 (initial_condition.f90:764-768)
    std::vector<double> dnux((size_t)n1 * n2, 0.0);
    if (P.iabsnb != 0 && std::fabs(in.xabsf - 1.0) > TINY) {
      const double x0 = P.xlen * in.xabsf, x2 = P.xlen - x0;
      for (int i1 = 0; i1 < n1; ++i1)
        if (c.cx[i1] >= x0)
          for (int i2 = 0; i2 < n2; ++i2) dnux[i1 + (size_t)n1 * i2] = in.coeffabsf * 2 * ((c.cx[i1] - x0) / x2);
    }
    d.dnux = upload(c, dnux);
    std::vector<double> dgz(n3), dre(std::max<size_t>(c.dposdy_ini.size(), 1)), dim(dre.size());
    for (int i3 = 0; i3 < n3; ++i3) dgz[i3] = dgzeddz_fn(P, c.cz[i3]);
    for (size_t i = 0; i < c.dposdy_ini.size(); ++i) {
      dre[i] = c.dposdy_ini[i].real();
      dim[i] = c.dposdy_ini[i].imag();
    }
    d.dgzed = upload(c, dgz);
    d.dposdy_re = upload(c, dre);
    d.dposdy_im = upload(c, dim);
    const size_t nw = std::max((size_t)n1 * n2, (size_t)n3a * n2);
    for (int i = 0; i < Dev::kW2; ++i) d.w2[i] = dalloc<double>(c, nw);
  }
  std::vector<double> pre(std::max<size_t>(c.pos_ini.size(), 1)), pim(pre.size());
  for (size_t i = 0; i < c.pos_ini.size(); ++i) { pre[i] = c.pos_ini[i].real(); pim[i] = c.pos_ini[i].imag(); }
  d.pos_re = upload(c, pre);
  d.pos_im = upload(c, pim);
  d.freq_w = upload(c, c.freq_w.empty() ? std::vector<double>(1, 0.0) : c.freq_w);
  d.gzed = upload(c, c.gzed);
  d.eiwt = dalloc<double>(c, 2 * (size_t)std::max(c.nf, 1));
  d.mat_coscos = upload(c, mat);
  d.probe_out = dalloc<double>(c, std::max(c.nprobes, 1));
  d.q_n1 = upload(c, quarter_table(n1 - 1));
  d.q_n2 = upload(c, quarter_table(std::max(n2 - 1, 1)));
  d.q_nd1 = upload(c, quarter_table(nd1 - 1));
  d.q_nd2 = upload(c, quarter_table(std::max(nd2 - 1, 1)));
  d.q_add = upload(c, quarter_table(n3a));
  if (n2 > 1) {
    // twiddle rows of the direct y passes (cos and sin kinds, n2 and nd2)
    for (int kind = 0; kind < 2; ++kind) {
      c.tb.ty_n2[kind] = upload(c, y_twiddle_rows(n2, kind == 1, &c.tb.ldy_n2));
      c.tb.ty_nd2[kind] = upload(c, y_twiddle_rows(nd2, kind == 1, &c.tb.ldy_nd2));
    }
  }
  c.tb.n1 = n1; c.tb.n2 = n2; c.tb.nd1 = nd1; c.tb.nd2 = nd2; c.tb.n3_add = n3a;
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c.tb.nsm = sms > 0 ? sms : 1;
    c.tb.part_cap = 64LL * 4 * c.tb.nsm * 16;   // partials of the split sums
    c.tb.cnt_cap = 4 * c.tb.nsm * 16;
    c.tb.part = dalloc<double>(c, (size_t)c.tb.part_cap);
    c.tb.cnt = dalloc<unsigned int>(c, (size_t)c.tb.cnt_cap);
    // two-level pass scratch: up to kMaxJobs x-pass jobs over nd2 lines,
    // B (A+1) 2 <= 2 (D+2) doubles per line for any factor pair
    c.tb.cs_cap = (long long)kMaxJobs * std::max(nd2, n2) * 4LL * (std::max(nd1, n1) + 2);
    c.tb.cs = dalloc<double>(c, (size_t)c.tb.cs_cap);
    // the wavemaker branch runs on its own stream with its own scratch
    c.tb2 = c.tb;
    c.tb2.part = dalloc<double>(c, (size_t)c.tb.part_cap);
    c.tb2.cnt = dalloc<unsigned int>(c, (size_t)c.tb.cnt_cap);
    c.tb2.cs = dalloc<double>(c, (size_t)c.tb.cs_cap);
    // and so does the eta-power branch
    c.tb3 = c.tb;
    c.tb3.part = dalloc<double>(c, (size_t)c.tb.part_cap);
    c.tb3.cnt = dalloc<unsigned int>(c, (size_t)c.tb.cnt_cap);
    c.tb3.cs = dalloc<double>(c, (size_t)c.tb.cs_cap);
  }
  c.tb.q_n1 = d.q_n1; c.tb.q_n2 = d.q_n2; c.tb.q_nd1 = d.q_nd1; c.tb.q_nd2 = d.q_nd2; c.tb.q_add = d.q_add;
  // FFT plans of the x and y lengths (passes over many lines: 3-D tanks)
  c.tb.nfft = 0;
  if (n2 > 1) {
    for (int D : {n1 - 1, n2 - 1, nd1 - 1, nd2 - 1}) {
      bool seen = false;
      for (int i = 0; i < c.tb.nfft; ++i) seen = seen || c.tb.fft[i].D == D;
      if (seen) continue;
      FftPlanInfo f;
      if (build_fft_plan(D, c.allocs, &f)) c.tb.fft[c.tb.nfft++] = f;
    }
  }
  for (Tables* t : {&c.tb2, &c.tb3}) {
    t->q_n1 = d.q_n1; t->q_n2 = d.q_n2; t->q_nd1 = d.q_nd1; t->q_nd2 = d.q_nd2; t->q_add = d.q_add;
    t->nfft = c.tb.nfft;
    for (int i = 0; i < c.tb.nfft; ++i) t->fft[i] = c.tb.fft[i];
  }
  for (void* p : c.allocs)
    if (!p) return fail(c, HOSNWT_ERR_CUDA, "device allocation failed");
  if (cudaGetLastError() != cudaSuccess) return fail(c, HOSNWT_ERR_CUDA, "upload failed");
  return HOSNWT_OK;
}

int alloc_device(Ctx& c) {
  const Params& P = c.P;
  Dev& d = c.d;
  const size_t nN = (size_t)P.n1 * P.n2, nB = (size_t)P.nd1 * P.nd2, nA = (size_t)P.n3a * P.n2;
  const size_t S = (size_t)c.L.size;
  const int M = P.M;
  if (cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess) return 1;
  d.y0 = dalloc<double>(c, S);
  d.ys = dalloc<double>(c, S);
  for (int s = 0; s < 5; ++s) d.k[s] = dalloc<double>(c, S);
  d.ynew = dalloc<double>(c, S);
  // eta, phis (and eta_c, phis_c) are adjacent, so that the drop-in step
  // moves them in one copy each way
  d.eta = dalloc<double>(c, 2 * nN);
  d.phis = d.eta + nN;
  d.eta_c = dalloc<double>(c, 2 * nN);
  d.phis_c = d.eta_c + nN;
  for (double** p : {&d.deta, &d.deta_c, &d.etam, &d.phim,
                     &d.eta_sp, &d.w_eta_x, &d.w_eta_y, &d.w_phi_x, &d.w_phi_y, &d.phix_add,
                     &d.phiy_add, &d.phiz_add, &d.phit_add, &d.phi_add, &d.phit_add1, &d.phiz_add1, &d.a1k,
                     &d.phiz1st, &d.rhs1, &d.X1, &d.X2, &d.X3, &d.det, &d.dph, &d.NL1, &d.NL2,
                     &d.pmode[0], &d.pmode[1], &d.pmode[2]})
    *p = dalloc<double>(c, nN);
  d.etapm.resize(M);
  d.phizm.assign(M + 2, nullptr);
  d.aHOS.assign(M + 2, nullptr);
  for (int j = 0; j < M; ++j) d.etapm[j] = dalloc<double>(c, nB);
  for (int j = 1; j <= M; ++j) { d.phizm[j] = dalloc<double>(c, nB); d.aHOS[j] = dalloc<double>(c, nB); }
  d.phizi.assign((size_t)M * M, nullptr);
  for (int m = 1; m <= M; ++m)
    for (int j = 1; j <= M + 1 - m; ++j) d.phizi[(m - 1) * M + (j - 1)] = dalloc<double>(c, nB);
  for (double** p : {&d.etax, &d.etay, &d.phisx, &d.phisy, &d.gradeta2, &d.phimext, &d.phizMm1,
                     &d.tbig, &d.tbig2, &d.ptmp, &d.pxe, &d.pye, &d.pze, &d.A1, &d.A3, &d.t1,
                     &d.geta2phiz, &d.geta2phiz2})
    *p = dalloc<double>(c, std::max(nB, nN));
  for (int g = 0; g < 24; ++g) d.grp[g] = dalloc<double>(c, std::max(nB, nN));
  for (int i = 0; i < Dev::kDealiasTmp; ++i) d.dtmp[i] = dalloc<double>(c, std::max(nB, nN));
  d.diag = dalloc<double>(c, 8);
  d.bc1 = dalloc<double>(c, nA);
  d.bcr = dalloc<double>(c, nA);
  if (P.n2 != 1) {
    const size_t nQ = (size_t)P.n1 * P.n3a * P.n2;
    for (int q = 0; q < 5; ++q) { d.Q[q] = dalloc<double>(c, nQ); d.B[q] = dalloc<double>(c, nQ); }
  }
  const size_t ntmp = (size_t)std::max(std::max(P.nd1, P.n3a), P.n1) * std::max(P.nd2, P.n2);
  for (int i = 0; i < kMaxJobs; ++i) {
    d.xtmp[i] = dalloc<double>(c, ntmp);
    d.xtmp2[i] = dalloc<double>(c, ntmp);
    d.xtmp3[i] = dalloc<double>(c, ntmp);
  }
  if (cudaStreamCreateWithFlags(&c.st2, cudaStreamNonBlocking) != cudaSuccess) return 1;
  if (cudaStreamCreateWithFlags(&c.st3, cudaStreamNonBlocking) != cudaSuccess) return 1;
  for (cudaEvent_t* e : {&c.ev_fork, &c.ev_eta, &c.ev_join, &c.ev_pow, &c.ev_acc, &c.ev_dl})
    if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return 1;
  for (cudaEvent_t& e : c.ev_pw)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return 1;
  d.sc = dalloc<double>(c, SC_COUNT);
  const size_t nparts = 10 * ((S + 255) / 256) + (std::max(nB, nN) + 63) / 64 + 1024;
  d.part = dalloc<double>(c, nparts);
  d.counter = dalloc<unsigned int>(c, 16);
  if (cudaMallocHost((void**)&d.host_sc, SC_COUNT * sizeof(double)) != cudaSuccess) return 1;
  std::memset(d.host_sc, 0, SC_COUNT * sizeof(double));
  // staging of the drop-in step: eta, phis, the eight arrays from a_add_1
  // on (their order in the state vector), and the error estimate
  if (cudaMallocHost((void**)&d.host_io, (2 * nN + (S - (size_t)c.L.off[S_AADD1]) + 1) * sizeof(double)) !=
      cudaSuccess)
    return 1;
  for (void* p : c.allocs)
    if (!p) return 1;
  return 0;
}

void free_device(Ctx& c) {
  if (c.ev0) cudaEventDestroy(c.ev0);
  if (c.ev1) cudaEventDestroy(c.ev1);
  c.ev0 = c.ev1 = nullptr;
  if (c.step_graph) cudaGraphExecDestroy(c.step_graph);
  c.step_graph = nullptr;
  if (c.loop_graph) cudaGraphExecDestroy(c.loop_graph);
  c.loop_graph = nullptr;
  if (c.ctl_dev) cudaFree(c.ctl_dev);
  c.ctl_dev = nullptr;
  if (c.ctl_host) cudaFreeHost(c.ctl_host);
  c.ctl_host = nullptr;
  for (void* p : c.allocs)
    if (p) cudaFree(p);
  c.allocs.clear();
  if (c.d.host_sc) cudaFreeHost(c.d.host_sc);
  c.d.host_sc = nullptr;
  if (c.d.host_io) cudaFreeHost(c.d.host_io);
  c.d.host_io = nullptr;
  for (cudaEvent_t e : {c.ev_fork, c.ev_eta, c.ev_join, c.ev_pow, c.ev_acc, c.ev_dl})
    if (e) cudaEventDestroy(e);
  c.ev_fork = c.ev_eta = c.ev_join = c.ev_pow = c.ev_acc = c.ev_dl = nullptr;
  for (cudaEvent_t& e : c.ev_pw) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  for (cudaStream_t* s : {&c.st2, &c.st3}) {
    if (*s) cudaStreamDestroy(*s);
    *s = nullptr;
  }
  if (c.st) cudaStreamDestroy(c.st);
  c.st = nullptr;
}

}  // namespace hos

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct hosnwt_ctx {
  hos::Ctx c;
};

static int cuda_check(Ctx& c, const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    c.err = std::string(what) + ": " + cudaGetErrorString(e);
    return HOSNWT_ERR_CUDA;
  }
  return HOSNWT_OK;
}

// Capture the step graph.  The first capture records the FFT batches that
// have no tuned layout yet; they are tuned on the stream (fft_tune_run) and
// the step is captured again with the tuned layouts.
static int build_step_graph(Ctx& c) {
  cudaGraph_t g = nullptr;
  for (int attempt = 0; attempt < 2; ++attempt) {
    const bool record = attempt == 0 && fft_tune_enabled();
    if (cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return cuda_check(c, "begin capture");
    cudaMemcpyAsync(c.d.sc + SC_T0, c.d.host_sc + SC_T0, 2 * sizeof(double), cudaMemcpyHostToDevice, c.st);
    const double f0 = g_xform_fmas;
    fft_tune_record(record);
    enqueue_step(c, c.st);
    fft_tune_record(false);
    c.fmas_per_step = g_xform_fmas - f0;
    if (cudaStreamEndCapture(c.st, &g) != cudaSuccess) return cuda_check(c, "end capture");
    if (!record) break;
    const int tuned = fft_tune_run(c.st);
    if (tuned < 0) {
      cudaGraphDestroy(g);
      return cuda_check(c, "FFT layout tuning");
    }
    if (tuned == 0) break;
    cudaGraphDestroy(g);
    g = nullptr;
  }
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  cudaGraphGetNodes(g, nodes.data(), &nn);
  c.kernels_per_step = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    cudaGraphNodeGetType(nd, &t);
    if (t == cudaGraphNodeTypeKernel) c.kernels_per_step++;
  }
  if (cudaGraphInstantiate(&c.step_graph, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_check(c, "graph instantiate");
  }
  cudaGraphDestroy(g);
  return HOSNWT_OK;
}

extern "C" int hosnwt_create(const hosnwt_input* in, const hosnwt_numerics* num, const char* wave_dir,
                             const double* probes_xy, int nprobes, hosnwt_ctx** out) {
  if (!in || !num || !out) return HOSNWT_ERR_ARG;
  *out = nullptr;
  hosnwt_ctx* h = new hosnwt_ctx();
  Ctx& c = h->c;
  c.in = *in;
  c.num = *num;
  int rc = setup(c, wave_dir, probes_xy, nprobes);
  if (rc == HOSNWT_OK) {
    // initial condition (initial_condition.f90:314-482)
    const size_t nN = (size_t)c.P.n1 * c.P.n2;
    std::vector<double> eta(nN, 0.0);
    if (c.P.icase == 1) {
      const double k1 = c.kx[c.P.islosh - 1];
      for (int i2 = 0; i2 < c.P.n2; ++i2)
        for (int i1 = 0; i1 < c.P.n1; ++i1) eta[i1 + (size_t)c.P.n1 * i2] = c.P.aslosh * std::cos(k1 * c.cx[i1]);
    }
    enqueue_initialize(c, c.st);
    cudaMemcpyAsync(c.d.eta, eta.data(), nN * sizeof(double), cudaMemcpyHostToDevice, c.st);
    cudaMemsetAsync(c.d.phis, 0, nN * sizeof(double), c.st);
    if (c.P.icase != 1) {
      // phi_add at t = 0 (initial_condition.f90:458-466: SWEET_1/2 and
      // phiadd_SL on the initial state): one right-hand side with dt = 0
      // into scratch slopes; the state is zero apart from the wavemaker
      // amplitudes, and the ramp and paddle position stay those of t = 0
      enqueue_set_scalar(c, SC_DT, 0.0, c.st);
      enqueue_rhs(c, c.d.y0, c.d.k[0], true, c.st);
      c.n_rhs = 0;
    }
    cudaStreamSynchronize(c.st);
    rc = cuda_check(c, "initialize");
    if (rc == HOSNWT_OK) rc = build_step_graph(c);
    c.time_cur = 0.0;
    c.endramp = 0;
  }
  if (rc != HOSNWT_OK) {
    // keep the context so the caller can read the message; it is unusable
    *out = h;
    return rc;
  }
  *out = h;
  return HOSNWT_OK;
}

extern "C" void hosnwt_destroy(hosnwt_ctx* h) {
  if (!h) return;
  free_device(h->c);
  delete h;
}

extern "C" const char* hosnwt_last_error(const hosnwt_ctx* h) { return h ? h->c.err.c_str() : "null context"; }

extern "C" int hosnwt_get_info(const hosnwt_ctx* h, hosnwt_info* info) {
  if (!h || !info) return HOSNWT_ERR_ARG;
  const Ctx& c = h->c;
  const Params& P = c.P;
  info->n1 = P.n1; info->n2 = P.n2; info->n3 = P.n3; info->n3_add = P.n3a;
  info->nd1 = P.nd1; info->nd2 = P.nd2; info->mHOS = P.M; info->p1 = P.p1; info->p2 = P.p2;
  info->Tscale = P.Tscale; info->xlen = P.xlen; info->ylen = P.ylen;
  info->dt_stab = P.dt_stab; info->delt = P.delt; info->delt_out = P.delt_out;
  info->T_stop = P.T_stop; info->toler = P.toler; info->time_cur = c.time_cur;
  info->nprobes = c.nprobes;
  info->n_rhs = c.n_rhs;
  info->kernels_per_step = c.kernels_per_step;
  info->device_ms = c.dev_ms;
  info->fmas_per_step = c.fmas_per_step;
  info->step_control = c.loop_state == 0 ? 0 : (c.loop_state < 0 ? 1 : (c.loop_pdl ? 2 : 3));
  return HOSNWT_OK;
}

static void timed_begin(Ctx& c) {
  if (!c.ev0) { cudaEventCreate(&c.ev0); cudaEventCreate(&c.ev1); }
  cudaEventRecord(c.ev0, c.st);
}
static void timed_end(Ctx& c) { cudaEventRecord(c.ev1, c.st); }
static void timed_collect(Ctx& c) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c.ev0, c.ev1) == cudaSuccess) c.dev_ms += ms;
}

// Launch one step graph; the error estimate lands in host_sc[SC_ERR] when
// the stream reaches it.
static int launch_step(Ctx& c, double t_o, double h_loc) {
  if (!c.step_graph) return HOSNWT_ERR_ARG;
  c.d.host_sc[SC_T0] = t_o;
  c.d.host_sc[SC_H] = h_loc;
  timed_begin(c);
  if (cudaGraphLaunch(c.step_graph, c.st) != cudaSuccess) return cuda_check(c, "graph launch");
  timed_end(c);
  cudaMemcpyAsync(c.d.host_sc + SC_ERR, c.d.sc + SC_ERR, sizeof(double), cudaMemcpyDeviceToHost, c.st);
  return HOSNWT_OK;
}

static int run_step(Ctx& c, double t_o, double h_loc, double* err) {
  const int rc = launch_step(c, t_o, h_loc);
  if (rc) return rc;
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return cuda_check(c, "step");
  timed_collect(c);
  c.n_rhs += 5;
  const double e = c.d.host_sc[SC_ERR];
  if (err) *err = e;
  if (!std::isfinite(e)) {
    c.err = "non-finite error estimate";
    return HOSNWT_ERR_NAN;
  }
  return HOSNWT_OK;
}

extern "C" int hosnwt_step(hosnwt_ctx* h, double h_loc, double* err) {
  if (!h || !(h_loc > 0.0)) return HOSNWT_ERR_ARG;
  return run_step(h->c, h->c.time_cur, h_loc, err);
}

extern "C" int hosnwt_accept(hosnwt_ctx* h, double h_loc) {
  if (!h) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const Params& P = c.P;
  bool end_ramp = false;
  if (P.iramp == 1 && P.Tramp - (c.time_cur + h_loc) <= TINY && P.Tramp > c.time_cur && c.endramp != 1) {
    end_ramp = true;
    c.endramp = 1;
  }
  timed_begin(c);
  enqueue_accept(c, end_ramp, c.st);
  timed_end(c);
  c.time_cur += h_loc;
  cudaStreamSynchronize(c.st);
  timed_collect(c);
  return cuda_check(c, "accept");
}

extern "C" int hosnwt_runge4_adapt2(hosnwt_ctx* h, double t_o, double* eta, double* phis,
                                    double* a_add_rk_1, double* a_add_rk_2, double* a_add_rkramp,
                                    double* a_add_rk_3, double* eta1st, double* eta2nd, double* a1st,
                                    double* a2nd, double h_loc, double* err) {
  if (!h || !eta || !phis || !a_add_rk_1 || !a_add_rk_2 || !a_add_rkramp || !a_add_rk_3 || !eta1st ||
      !eta2nd || !a1st || !a2nd || !err)
    return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const StateLayout& L = c.L;
  const size_t nN = (size_t)c.P.n1 * c.P.n2, nA = (size_t)c.P.n3a * c.P.n2;
  double* const arr[10] = {eta, phis, a_add_rk_1, a_add_rk_2, a_add_rkramp, a_add_rk_3, a1st, eta1st, a2nd, eta2nd};
  const size_t sz[10] = {nN, nN, nA, nA, nA, nA, nN, nN, nN, nN};
  // one pinned staging buffer, two copies each way, one synchronisation:
  // [eta | phis] and the state vector from a_add_1 on are contiguous on the
  // device, in the order of the arguments
  double* io = c.d.host_io;
  size_t o = 0;
  for (int a = 0; a < 10; ++a) {
    std::memcpy(io + o, arr[a], sz[a] * sizeof(double));
    o += sz[a];
  }
  const size_t ntail = o - 2 * nN;
  cudaMemcpyAsync(c.d.eta, io, 2 * nN * sizeof(double), cudaMemcpyHostToDevice, c.st);
  cudaMemcpyAsync(c.d.y0 + L.off[S_AADD1], io + 2 * nN, ntail * sizeof(double), cudaMemcpyHostToDevice, c.st);
  int rc = launch_step(c, t_o, h_loc);
  if (rc) return rc;
  cudaMemcpyAsync(io, c.d.eta_c, 2 * nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaMemcpyAsync(io + 2 * nN, c.d.ynew + L.off[S_AADD1], ntail * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return cuda_check(c, "runge4_adapt2");
  timed_collect(c);
  c.n_rhs += 5;
  o = 0;
  for (int a = 0; a < 10; ++a) {
    std::memcpy(arr[a], io + o, sz[a] * sizeof(double));
    o += sz[a];
  }
  const double e = c.d.host_sc[SC_ERR];
  *err = e;
  if (!std::isfinite(e)) {
    c.err = "non-finite error estimate";
    rc = HOSNWT_ERR_NAN;
  }
  const int rc2 = cuda_check(c, "runge4_adapt2");
  return rc2 ? rc2 : rc;
}

// step control (HOS-NWT.f90:498-571)
static int advance(Ctx& c, double time_next, double* h_rk_io, int* n_acc, int* n_rej) {
  const Params& P = c.P;
  double h_rk = *h_rk_io;
  int na = 0, nr = 0;
  while (c.time_cur < time_next) {
    double h_loc = h_rk;
    if (time_next - c.time_cur < h_rk) h_loc = time_next - c.time_cur;
    double error = 0.0;
    int rc = run_step(c, c.time_cur, h_loc, &error);
    if (rc) return rc;
    double dt_correc;
    if (error > P.toler && h_rk > 0.001 * 0.95 * P.dt_stab) {
      // REAL(4) constants of the reference (HOS-NWT.f90:525)
      dt_correc = (double)0.9f * std::pow(error / P.toler, -(double)(1.0f / 4.0f));
      nr++;
      if (std::fabs(P.Tramp - (c.time_cur + h_loc)) <= TINY && P.Tramp > c.time_cur) c.endramp = 0;
    } else {
      bool end_ramp = false;
      if (P.iramp == 1 && P.Tramp - (c.time_cur + h_loc) <= TINY && P.Tramp > c.time_cur && c.endramp != 1) {
        end_ramp = true;
        c.endramp = 1;
      }
      enqueue_accept(c, end_ramp, c.st);
      c.time_cur = c.time_cur + h_loc;
      dt_correc = std::fabs(error) < TINY ? 2.0 : 0.9 * std::pow(error / P.toler, -(1.0 / 4.0));
      na++;
    }
    h_rk = h_rk * dt_correc;
    h_rk = std::min(std::min(h_rk, 0.95 * P.dt_stab), P.delt_out);
    h_rk = std::max(std::max(h_rk, 0.0001 * 0.95 * P.dt_stab), 0.0001 * P.delt_out);
  }
  cudaStreamSynchronize(c.st);
  *h_rk_io = h_rk;
  if (n_acc) *n_acc = na;
  if (n_rej) *n_rej = nr;
  return cuda_check(c, "advance");
}

// ---------------------------------------------------------------------------
// Step control on the device.  An output interval runs as one graph:
//   copy the control block in -> WHILE { k_ctl_begin, the RK4(5) step,
//   k_ctl_end (decision, loop condition), k_accept_ctl } -> copy it out
// so that the host waits once per interval instead of once per step.
// HOSNWT_DEVICE_LOOP=0 keeps the host loop of advance().
// ---------------------------------------------------------------------------
static bool device_loop_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("HOSNWT_DEVICE_LOOP");
    return !(e && e[0] == '0');
  }();
  return on;
}

static const int kMaxLoopSteps = 1 << 24;  // attempted steps per interval before the loop stops

// Capture the body into the WHILE node of a fresh graph and instantiate it.
static bool try_build_loop(Ctx& c, bool pdl) {
  const Params& P = c.P;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  bool ok = false;
  do {
    cudaGraphConditionalHandle cond;
    if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) break;
    cudaGraphNode_t n_in = nullptr, n_loop = nullptr, n_out = nullptr;
    if (cudaGraphAddMemcpyNode1D(&n_in, g, nullptr, 0, c.ctl_dev, c.ctl_host, sizeof(StepCtl),
                                 cudaMemcpyHostToDevice) != cudaSuccess)
      break;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    if (cudaGraphAddNode(&n_loop, g, &n_in, nullptr, 1, &np) != cudaSuccess) break;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    CtlParams cp{};
    cp.toler = P.toler;
    cp.dt_stab = P.dt_stab;
    cp.delt_out = P.delt_out;
    cp.Tramp = P.Tramp;
    cp.iramp = P.iramp;
    cp.max_iters = kMaxLoopSteps;
    cp.cond = cond;
    if (cudaStreamBeginCaptureToGraph(c.st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess)
      break;
    g_launch_no_pdl = !pdl;
    const double f0 = g_xform_fmas;
    enqueue_ctl_step(c, c.ctl_dev, cp, c.st);
    g_xform_fmas = f0;
    g_launch_no_pdl = false;
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(c.st, &captured) != cudaSuccess) break;
    if (cudaGraphAddMemcpyNode1D(&n_out, g, &n_loop, 1, c.ctl_host, c.ctl_dev, sizeof(StepCtl),
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
      break;
    if (cudaGraphInstantiate(&c.loop_graph, g, 0) != cudaSuccess) {
      c.loop_graph = nullptr;
      break;
    }
    ok = true;
  } while (false);
  g_launch_no_pdl = false;
  cudaGraphDestroy(g);
  (void)cudaGetLastError();  // a failed attempt leaves no error behind
  return ok;
}

// Build the loop graph on first use: with programmatic dependencies inside
// the body if the runtime accepts them there, else fully serialised; -1
// (the host loop) if neither builds.
static void ensure_loop(Ctx& c) {
  if (c.loop_state != 0) return;
  c.loop_state = -1;
  if (!device_loop_enabled() || !c.step_graph) return;
  if (!c.ctl_dev && cudaMalloc((void**)&c.ctl_dev, sizeof(StepCtl)) != cudaSuccess) {
    c.ctl_dev = nullptr;
    (void)cudaGetLastError();
    return;
  }
  if (!c.ctl_host && cudaMallocHost((void**)&c.ctl_host, sizeof(StepCtl)) != cudaSuccess) {
    c.ctl_host = nullptr;
    (void)cudaGetLastError();
    return;
  }
  if (try_build_loop(c, true)) {
    c.loop_state = 1;
    c.loop_pdl = true;
  } else if (try_build_loop(c, false)) {
    c.loop_state = 1;
    c.loop_pdl = false;
  }
}

// Launch one interval of the device loop (the host's h_rk, time_cur and
// endramp go in through the pinned block); finish_loop collects it.
static int launch_loop(Ctx& c, double time_next, double h_rk) {
  StepCtl& b = *c.ctl_host;
  std::memset(&b, 0, sizeof(StepCtl));
  b.time_cur = c.time_cur;
  b.h_rk = h_rk;
  b.time_next = time_next;
  b.endramp = c.endramp;
  timed_begin(c);
  if (cudaGraphLaunch(c.loop_graph, c.st) != cudaSuccess) return cuda_check(c, "loop graph launch");
  timed_end(c);
  return HOSNWT_OK;
}

static int finish_loop(Ctx& c, double* h_rk_io, int* n_acc, int* n_rej) {
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return cuda_check(c, "advance");
  timed_collect(c);
  const StepCtl& b = *c.ctl_host;
  c.n_rhs += 5LL * b.iters;
  c.time_cur = b.time_cur;
  c.endramp = b.endramp;
  *h_rk_io = b.h_rk;
  if (n_acc) *n_acc = b.n_acc;
  if (n_rej) *n_rej = b.n_rej;
  if (b.status == 1) {
    c.err = "non-finite error estimate";
    return HOSNWT_ERR_NAN;
  }
  if (b.status == 2) return fail(c, HOSNWT_ERR_DT_UNDERFLOW, "more than %d attempted steps in one interval",
                                 kMaxLoopSteps);
  return cuda_check(c, "advance");
}

static int advance_any(Ctx& c, double time_next, double* h_rk_io, int* n_acc, int* n_rej) {
  ensure_loop(c);
  if (c.loop_state != 1) return advance(c, time_next, h_rk_io, n_acc, n_rej);
  if (!(c.time_cur < time_next)) {
    if (n_acc) *n_acc = 0;
    if (n_rej) *n_rej = 0;
    return HOSNWT_OK;
  }
  const int rc = launch_loop(c, time_next, *h_rk_io);
  if (rc) return rc;
  return finish_loop(c, h_rk_io, n_acc, n_rej);
}

extern "C" int hosnwt_advance(hosnwt_ctx* h, double time_next, double* h_rk, int* n_acc, int* n_rej) {
  if (!h || !h_rk) return HOSNWT_ERR_ARG;
  return advance_any(h->c, time_next, h_rk, n_acc, n_rej);
}

extern "C" int hosnwt_probes(hosnwt_ctx* h, double* out) {
  if (!h || !out) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  if (c.nprobes <= 0) return HOSNWT_OK;
  enqueue_probes(c, c.st);
  cudaMemcpyAsync(out, c.d.probe_out, c.nprobes * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "probes");
}

// ---------------------------------------------------------------------------
// output files (output.f90:37-229, 232-482) and diagnostics
// ---------------------------------------------------------------------------
// Fortran Ew.d / Dw.d: 0.ddddd x 10^e, right-justified in w
static std::string fortran_E(double v, int w, int d, char letter) {
  char buf[64];
  std::string body;
  if (v == 0.0 || !std::isfinite(v)) {
    body = "0." + std::string(d, '0') + letter + "+00";
    if (!std::isfinite(v)) body = std::string(w, '*');
  } else {
    std::snprintf(buf, sizeof buf, "%.*E", d - 1, std::fabs(v));
    std::string t(buf);  // x.xxxxE+yy
    const size_t ep = t.find('E');
    std::string digits = t.substr(0, 1) + t.substr(2, ep - 2);
    int e = std::atoi(t.c_str() + ep + 1) + 1;
    std::snprintf(buf, sizeof buf, "%c%02d", e < 0 ? '-' : '+', std::abs(e));
    body = std::string(v < 0 ? "-" : "") + "0." + digits + letter + buf;
  }
  if ((int)body.size() < w) body = std::string(w - body.size(), ' ') + body;
  return body;
}

static std::string fortran_ES(double v, int w, int d) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%*.*E", w, d, v);
  return buf;
}

// Fortran Fw.d and Iw: asterisks when the value does not fit in w
static std::string fortran_F(double v, int w, int d) {
  char buf[64];
  const int n = std::snprintf(buf, sizeof buf, "%*.*f", w, d, v);
  if (n > w || !std::isfinite(v)) return std::string(w, '*');
  return buf;
}
static std::string fortran_I(long long v, int w) {
  char buf[32];
  const int n = std::snprintf(buf, sizeof buf, "%*lld", w, v);
  if (n > w) return std::string(w, '*');
  return buf;
}

static std::string rjust(const std::string& s, size_t w) {
  if (s.size() >= w) return s.substr(0, w);
  return std::string(w - s.size(), ' ') + s;
}

// write_input (input.f90:318-395): the input echo at the top of each result file
static void write_input(FILE* f, const Ctx& c) {
  const hosnwt_input& in = c.in;
  auto blank = [&](const char* t) { std::fprintf(f, "#%s\n", t); };
  auto R = [&](double v, const char* var, const char* txt) {
    std::fprintf(f, "#%s:: %s:: %s\n", rjust(txt, 33).c_str(), rjust(var, 13).c_str(), fortran_ES(v, 25, 16).c_str());
  };
  auto I = [&](int v, const char* var, const char* txt) {
    std::fprintf(f, "#%s:: %s:: %5d\n", rjust(txt, 33).c_str(), rjust(var, 13).c_str(), v);
  };
  auto A = [&](const char* v, const char* var, const char* txt) {
    std::fprintf(f, "#%s:: %s:: %s\n", rjust(txt, 33).c_str(), rjust(var, 13).c_str(), v);
  };
  blank("----------------------- Tank dimensions -----------------------");
  R(in.xlen, "xlen", "Length(m) of the wavetank");
  R(in.ylen, "ylen", "Beam(m) of the wavetank");
  R(in.h, "h", "Depth(m) of the wavetank");
  blank("------------------------ Select case --------------------------");
  I(in.icase, "icase", "Choice of computed case");
  blank("------------------ Sloshing case (icase = 1) ------------------");
  I(in.islosh + 1, "islosh", "Number of the natural mode");
  R(in.aslosh, "aslosh", "Amplitude (m) of the mode");
  blank("--------------- Monochromatic case (icase = 2) ----------------");
  R(in.amp_mono, "amp_mono", "Amplitude (m) of wave train");
  R(in.nu_mono, "nu_mono", "Frequency (Hz) of wave train");
  R(c.P.theta_mono, "theta_mono", "Angle (deg) from x-axis");
  R(in.ph_mono, "ph_mono", "Phasis (rad) of wave train");
  I(in.ibat, "ibat", "Directional wmk type");
  R(in.xd_mono, "xd_mono", "Wave target distance (ibat=3)");
  blank("-------------------- File case (icase = 3) --------------------");
  A(in.file_name, "file_name", "Name of frequency file");
  I(in.i_cut, "i_cut", "Frequency cut-off");
  R(in.nuc_low, "nuc_low", "Low cut_off frequency (Hz)");
  R(in.nuc_high, "nuc_high", "High cut_off frequency (Hz) ");
  blank("------------------ Irregular wave (icase=4) -------------------");
  R(in.Hs, "Hs", "Significant wave height (m)");
  R(in.Tp, "Tp", "Peak period (s)");
  R(in.gamma, "gamma", "Shape factor (Jonswap)");
  I(in.iseed, "iseed", "Seed number for random numb. ");
  blank("-------------------- Wavemaker definition ---------------------");
  I(in.i_wmk, "i_wmk", "Nonlinear order of wavemaker");
  I(in.igeom, "igeom", "Type (1: piston, 2: hinged)");
  R(in.d_hinge, "d_hinge", "Rotation axis distance");
  I(in.iramp, "iramp", "Time ramp");
  R(in.iramp == 0 ? 0.0 : in.Tramp, "Tramp", "Time ramp duration");
  blank("----------------------- Numerical beach -----------------------");
  I(in.iabsnb, "iabsnb", "Absorption numerical beach");
  R(in.xabsf, "xabsf", "Beginning front num. beach");
  R(in.coeffabsf, "coeffabsf", "Absorption strength front");
  blank("------------- Elevation/Velocity-Pressure probes --------------");
  I(in.iprobes, "iprobes", "Use of probes");
  A(in.pro_file, "pro_file", "Filename of probe positions");
  blank("---------------------- Time-integration -----------------------");
  R(in.T_stop, "T_stop", "Duration of the simulation");
  R(in.toler, "toler", "Time tolerance: RK 4(5)");
  R(in.f_out, "f_out", "Output frequency");
  blank("--------------------------- Output ----------------------------");
  I(in.idim, "idim", "Output: 1-dim. ; 0-nondim.");
  I(in.i3d, "i3d", "Free surface plot");
  I(in.imodes, "imodes", "Modes plot");
  I(in.iwmk, "iwmk", "Wavemaker motion plot");
  I(in.i_sw, "i_sw", "Swense output 1='yes',0='no'");
  blank("--------------------- Numerical parameters ---------------------");
  I(c.P.n1, "n1", "Number of nodes/modes in x");
  I(c.P.n2, "n2", "Number of nodes/modes in y");
  I(c.P.n3, "n3", "Number of nodes/modes on wmk");
  I(c.P.M, "mHOS", "HOS order");
  I(c.P.p1, "p1", "Dealiasing in x-direction");
  I(c.P.p2, "p2", "Dealiasing in y-direction");
  R(1.0, "coeffilt(1)", "Filtering ratio in x-modes");
  R(1.0, "coeffilt(2)", "Filtering ratio in y-modes");
  R(1.0, "coeffilt(3)", "Filtering ratio in z-modes");
}

// volume, energies and slopes of the current state (vol_energy.f90:36-119)
static int diagnostics(Ctx& c, double out[5]) {
  enqueue_diagnostics(c, c.d.diag, c.st);
  double raw[5];
  cudaMemcpyAsync(raw, c.d.diag, 5 * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return cuda_check(c, "diagnostics");
  const Params& P = c.P;
  double vol = raw[0] * P.delx / P.xlen, ep = raw[1] * P.delx / 2.0, ek = raw[2] * P.delx / 2.0;
  if (P.n2 != 1) {
    vol = vol / P.ylen * P.dely;
    ep *= P.dely;
    ek *= P.dely;
  }
  out[0] = vol;
  out[1] = ep;
  out[2] = ek;
  out[3] = raw[3];
  out[4] = raw[4];
  return HOSNWT_OK;
}

// check_slope (initial_condition.f90:687-716): filter eta and phis when the
// slope of the last right-hand side exceeds 8
static int check_slope(Ctx& c, int* filtered) {
  double dg[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  int rc = diagnostics(c, dg);
  if (rc) return rc;
  int f = 0;
  if (dg[3] > 8.0) { enqueue_slope_filter(c, 0, c.st); f |= 1; }
  if (dg[4] > 8.0 && c.P.n2 != 1) { enqueue_slope_filter(c, 1, c.st); f |= 2; }
  if (filtered) *filtered = f;
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "check_slope");
}

extern "C" int hosnwt_diagnostics(hosnwt_ctx* h, double* out5) {
  if (!h || !out5) return HOSNWT_ERR_ARG;
  return diagnostics(h->c, out5);
}

extern "C" int hosnwt_check_slope(hosnwt_ctx* h, int* filtered) {
  if (!h) return HOSNWT_ERR_ARG;
  return check_slope(h->c, filtered);
}

extern "C" int hosnwt_run(hosnwt_ctx* h, const char* results_dir) {
  if (!h) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const Params& P = c.P;
  const bool dimensional = c.in.idim == 1;
  const double t_adim = dimensional ? P.Tscale : 1.0, x_adim = dimensional ? P.h : 1.0;
  FILE* fp = nullptr;
  FILE* fv = nullptr;
  if (results_dir) {
    std::string path = std::string(results_dir) + "/probes.dat";
    if (c.nprobes > 0) {
      fp = std::fopen(path.c_str(), "w");
      if (!fp) return fail(c, HOSNWT_ERR_IO, "cannot open %s", path.c_str());
      write_input(fp, c);
      std::fprintf(fp, "TITLE=\"Probes elevation records versus time\"\n");
      std::fprintf(fp, dimensional ? "VARIABLES = \"time\" " : "VARIABLES = \"time*sqrt(g/h)\" ");
      for (int p = 0; p < c.nprobes; ++p) std::fprintf(fp, dimensional ? "\"p%d\" " : "\"p%d/h\" ", p + 1);
      std::fprintf(fp, "\n");
    }
    path = std::string(results_dir) + "/vol_energy.dat";
    fv = std::fopen(path.c_str(), "w");
    if (!fv) {
      if (fp) std::fclose(fp);
      return fail(c, HOSNWT_ERR_IO, "cannot open %s", path.c_str());
    }
    write_input(fv, c);
    std::fprintf(fv, "TITLE=\" volume and energy evolution \"\n");
    std::fprintf(fv, dimensional ? "VARIABLES=\"time\", \"voltot\", \"enepot\", \"enekin\", \"enetot\"\n"
                                 : "VARIABLES=\"time*sqrt(g/h)\", \"voltot\", \"enepot\", \"enekin\", \"enetot\"\n");
  }
  // 3d.dat (i3d = 1): free-surface zones (output.f90:47-56, 291-345)
  FILE* f3 = nullptr;
  if (results_dir && c.in.i3d == 1) {
    const std::string path = std::string(results_dir) + "/3d.dat";
    f3 = std::fopen(path.c_str(), "w");
    if (!f3) {
      if (fp) std::fclose(fp);
      if (fv) std::fclose(fv);
      return fail(c, HOSNWT_ERR_IO, "cannot open %s", path.c_str());
    }
    write_input(f3, c);
    std::fprintf(f3, " TITLE=\" 3D free surface elevation \"\n");
    std::fprintf(f3, dimensional ? "VARIABLES=\"x\",\"y\",\"eta\",\"phis\"\n"
                                 : "VARIABLES=\"x/h\",\"y/h\",\"eta/h\",\"phis*sqrt(h/g)/h**2\"\n");
  }
  const size_t nN = (size_t)P.n1 * P.n2;
  std::vector<double> eta_h, phis_h;
  auto write_3d = [&]() {
    eta_h.resize(nN);
    phis_h.resize(nN);
    cudaMemcpy(eta_h.data(), c.d.eta, nN * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(phis_h.data(), c.d.phis, nN * sizeof(double), cudaMemcpyDeviceToHost);
    const bool first = std::fabs(c.time_cur) < TINY;
    std::fprintf(f3, "ZONE SOLUTIONTIME = %s%s I=%s, J=%s\n", fortran_F(c.time_cur * t_adim, 6, 2).c_str(),
                 first ? "," : ", D=(1,2),", fortran_I(P.n1, 4).c_str(), fortran_I(P.n2, 4).c_str());
    for (int i2 = 0; i2 < P.n2; ++i2)
      for (int i1 = 0; i1 < P.n1; ++i1) {
        const size_t i = i1 + (size_t)P.n1 * i2;
        if (first) {
          std::fprintf(f3, "%s %s %s %s \n", fortran_F(c.cx[i1] * x_adim, 10, 5).c_str(),
                       fortran_F(c.cy[i2] * x_adim, 10, 5).c_str(), fortran_ES(eta_h[i] * x_adim, 12, 5).c_str(),
                       fortran_ES(phis_h[i] * x_adim * x_adim / t_adim, 12, 5).c_str());
        } else {
          double target = 0.0;
          if (P.icase == 2 && (P.igeom == 1 || P.igeom == 2))
            target = P.amp_mono * std::cos(P.w_mono * c.time_cur -
                                           c.k_mono * (c.cx[i1] * std::cos(P.theta_mono) +
                                                       c.cy[i2] * std::sin(P.theta_mono)) +
                                           P.ph_mono);
          std::fprintf(f3, "%s %s \n", fortran_ES(eta_h[i] * x_adim, 12, 5).c_str(),
                       fortran_ES((eta_h[i] - target) * x_adim, 12, 5).c_str());
        }
      }
  };
  std::vector<double> pv(std::max(c.nprobes, 1));
  double delt = P.delt;
  int rc = HOSNWT_OK;
  while (c.time_cur < P.T_stop + P.delt_out) {
    if (f3) write_3d();
    if (fv) {
      // output_time_step (output.f90:232-282)
      double dg[5];
      rc = diagnostics(c, dg);
      if (rc) break;
      double sc[SC_COUNT];
      cudaMemcpy(sc, c.d.sc, sizeof sc, cudaMemcpyDeviceToHost);
      double eta11 = 0.0;
      cudaMemcpy(&eta11, c.d.eta, sizeof(double), cudaMemcpyDeviceToHost);
      double vol = dg[0];
      const double a = sc[SC_ALPHA], pt = sc[SC_POSTOP];
      if (P.igeom == 2) vol = vol - 0.5 * a * (1 - P.d_hinge) * pt / P.xlen - eta11 * a * pt / P.xlen;
      else if (P.igeom == 1) vol = vol - a * pt / P.xlen - eta11 * a * pt / P.xlen;
      std::fprintf(fv, "%s %s %s %s %s \n", fortran_ES(c.time_cur * t_adim, 12, 5).c_str(),
                   fortran_ES(vol, 12, 5).c_str(), fortran_ES(dg[1], 12, 5).c_str(),
                   fortran_ES(dg[2], 12, 5).c_str(), fortran_ES(dg[1] + dg[2], 12, 5).c_str());
    }
    if (fp) {
      rc = hosnwt_probes(h, pv.data());
      if (rc) break;
      std::string line = fortran_E(c.time_cur * t_adim, 13, 5, 'D');
      for (int p = 0; p < c.nprobes; ++p) line += fortran_E(pv[p] * x_adim, 13, 5, 'D');
      std::fprintf(fp, "%s\n", line.c_str());
    }
    if (std::fabs(c.time_cur - P.T_stop) <= TINY) break;
    double time_next = c.time_cur + P.delt_out;
    if (time_next > P.T_stop + P.delt_out) time_next = P.T_stop + P.delt_out;
    double h_rk = delt;
    rc = advance_any(c, time_next, &h_rk, nullptr, nullptr);
    if (rc) break;
    delt = h_rk;
    rc = check_slope(c, nullptr);
    if (rc) break;
  }
  if (fp) std::fclose(fp);
  if (fv) std::fclose(fv);
  if (f3) std::fclose(f3);
  return rc;
}

extern "C" int hosnwt_get_state(hosnwt_ctx* h, double* eta, double* phis, double* deta) {
  if (!h) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const size_t nN = (size_t)c.P.n1 * c.P.n2;
  if (eta) cudaMemcpyAsync(eta, c.d.eta, nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  if (phis) cudaMemcpyAsync(phis, c.d.phis, nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  if (deta) cudaMemcpyAsync(deta, c.d.deta, nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "get_state");
}

extern "C" int hosnwt_get_rk_state(hosnwt_ctx* h, double* eta, double* phis, double* a_add_1,
                                   double* a_add_2, double* a_add_ramp, double* a_add_3,
                                   double* eta1st, double* eta2nd, double* a1st, double* a2nd) {
  if (!h || !eta || !phis || !a_add_1 || !a_add_2 || !a_add_ramp || !a_add_3 || !eta1st || !eta2nd ||
      !a1st || !a2nd)
    return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const StateLayout& L = c.L;
  const size_t nN = (size_t)c.P.n1 * c.P.n2, nA = (size_t)c.P.n3a * c.P.n2;
  double* const arr[10] = {nullptr, nullptr, a_add_1, a_add_2, a_add_ramp, a_add_3, a1st, eta1st, a2nd, eta2nd};
  const size_t sz[10] = {nN, nN, nA, nA, nA, nA, nN, nN, nN, nN};
  cudaMemcpyAsync(eta, c.d.eta, nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaMemcpyAsync(phis, c.d.phis, nN * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  for (int a = 2; a < 10; ++a)
    cudaMemcpyAsync(arr[a], c.d.y0 + L.off[a], sz[a] * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "get_rk_state");
}

extern "C" int hosnwt_set_state(hosnwt_ctx* h, const double* eta, const double* phis) {
  if (!h) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const size_t nN = (size_t)c.P.n1 * c.P.n2;
  if (eta) cudaMemcpyAsync(c.d.eta, eta, nN * sizeof(double), cudaMemcpyHostToDevice, c.st);
  if (phis) cudaMemcpyAsync(c.d.phis, phis, nN * sizeof(double), cudaMemcpyHostToDevice, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "set_state");
}

extern "C" int hosnwt_solveHOS2(hosnwt_ctx* h, const double* const* y, double* const* k, double delta_t,
                                double time, double alpha_prev, double pos_top_prev) {
  if (!h || !y || !k) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const StateLayout& L = c.L;
  const size_t nN = (size_t)c.P.n1 * c.P.n2, nA = (size_t)c.P.n3a * c.P.n2;
  const size_t sz[10] = {nN, nN, nA, nA, nA, nA, nN, nN, nN, nN};
  for (int a = 0; a < 10; ++a) {
    if (!y[a] || !k[a]) return HOSNWT_ERR_ARG;
    cudaMemcpyAsync(c.d.ys + L.off[a], y[a], sz[a] * sizeof(double), cudaMemcpyHostToDevice, c.st);
  }
  enqueue_set_scalar(c, SC_DT, delta_t, c.st);
  enqueue_set_scalar(c, SC_TIME, time, c.st);
  enqueue_set_scalar(c, SC_ALPHA, alpha_prev, c.st);
  enqueue_set_scalar(c, SC_POSTOP, pos_top_prev, c.st);
  enqueue_rhs(c, c.d.ys, c.d.k[0], false, c.st);
  for (int a = 0; a < 10; ++a)
    cudaMemcpyAsync(k[a], c.d.k[0] + L.off[a], sz[a] * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "solveHOS2");
}

extern "C" int hosnwt_hos_terms(hosnwt_ctx* h, double* eta_big, double* phizm) {
  if (!h || !eta_big || !phizm) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const size_t nB = (size_t)c.P.nd1 * c.P.nd2;
  if (c.n_rhs == 0) return fail(c, HOSNWT_ERR_ARG, "hos_terms: no right-hand side has been evaluated");
  // the scratch fields of the last right-hand side enqueued on this context
  cudaStreamSynchronize(c.st);
  cudaMemcpyAsync(eta_big, c.d.etapm[0], nB * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  for (int m = 1; m <= c.P.M; ++m)
    cudaMemcpyAsync(phizm + (size_t)(m - 1) * nB, c.d.phizm[m], nB * sizeof(double), cudaMemcpyDeviceToHost,
                    c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "hos_terms");
}

extern "C" int hosnwt_transform(hosnwt_ctx* h, int grid, int dir, int csx, int csy, const double* in,
                                double* out) {
  if (!h || !in || !out || grid < 0 || grid > 2 || (dir != 1 && dir != -1)) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const Params& P = c.P;
  int a = P.n1, b = P.n2;
  if (grid == GRID_BIG) { a = P.nd1; b = P.nd2; }
  else if (grid == GRID_ADD) { a = P.n3a; b = P.n2; }
  const size_t n = (size_t)a * b;
  cudaMemcpyAsync(c.d.tbig, in, n * sizeof(double), cudaMemcpyHostToDevice, c.st);
  XfReq r;
  r.grid = grid; r.dir = dir; r.csx = csx; r.csy = csy;
  r.in = c.d.tbig; r.in_ld = a; r.nin1 = a; r.nin2 = b;
  r.out = c.d.tbig2; r.out_ld = a; r.nout1 = a; r.nout2 = b;
  r.scale = 1.0;
  launch_transforms(&r, 1, c.tb, c.d.xtmp, c.st);
  cudaMemcpyAsync(out, c.d.tbig2, n * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return cuda_check(c, "transform");
}

extern "C" int hosnwt_advance_many(hosnwt_ctx* const* ctxs, int n, const double* time_next, double* h_rk) {
  if (!ctxs || n <= 0 || !time_next || !h_rk) return HOSNWT_ERR_ARG;
  // The device-controlled loop of hosnwt_advance (one graph launch per tank
  // and interval) was measured slower here: 64 tanks advanced 1 s each took
  // 18.2 s with every tank's loop graph in flight at once, 15.2 s with the
  // per-step relaunch below.
  // Independent tanks, each on its own stream with its own step graph and
  // the step control of HOS-NWT.f90:498-571.  Each tank is relaunched as
  // soon as its own step has finished (polled with an event), so tanks of
  // different sizes overlap on the GPU without waiting for each other.
  std::vector<double> h_loc(n, 0.0);
  std::vector<char> inflight(n, 0);
  std::vector<cudaEvent_t> done(n, nullptr);
  int rc = HOSNWT_OK;
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i] || !ctxs[i]->c.step_graph) return HOSNWT_ERR_ARG;
    cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
  }
  auto launch = [&](int i) -> int {
    Ctx& c = ctxs[i]->c;
    h_loc[i] = h_rk[i];
    if (time_next[i] - c.time_cur < h_rk[i]) h_loc[i] = time_next[i] - c.time_cur;
    c.d.host_sc[SC_T0] = c.time_cur;
    c.d.host_sc[SC_H] = h_loc[i];
    if (cudaGraphLaunch(c.step_graph, c.st) != cudaSuccess) return cuda_check(c, "graph launch");
    cudaMemcpyAsync(c.d.host_sc + SC_ERR, c.d.sc + SC_ERR, sizeof(double), cudaMemcpyDeviceToHost, c.st);
    cudaEventRecord(done[i], c.st);
    inflight[i] = 1;
    return HOSNWT_OK;
  };
  int running = 0;
  for (int i = 0; i < n && rc == HOSNWT_OK; ++i)
    if (ctxs[i]->c.time_cur < time_next[i]) {
      rc = launch(i);
      ++running;
    }
  while (running > 0 && rc == HOSNWT_OK) {
    for (int i = 0; i < n && rc == HOSNWT_OK; ++i) {
      if (!inflight[i]) continue;
      const cudaError_t q = cudaEventQuery(done[i]);
      if (q == cudaErrorNotReady) continue;
      Ctx& c = ctxs[i]->c;
      const Params& P = c.P;
      inflight[i] = 0;
      if (q != cudaSuccess) { rc = cuda_check(c, "step"); break; }
      c.n_rhs += 5;
      const double error = c.d.host_sc[SC_ERR];
      if (!std::isfinite(error)) {
        c.err = "non-finite error estimate";
        rc = HOSNWT_ERR_NAN;
        break;
      }
      double dt_correc;
      if (error > P.toler && h_rk[i] > 0.001 * 0.95 * P.dt_stab) {
        dt_correc = (double)0.9f * std::pow(error / P.toler, -(double)(1.0f / 4.0f));
        if (std::fabs(P.Tramp - (c.time_cur + h_loc[i])) <= TINY && P.Tramp > c.time_cur) c.endramp = 0;
      } else {
        bool end_ramp = false;
        if (P.iramp == 1 && P.Tramp - (c.time_cur + h_loc[i]) <= TINY && P.Tramp > c.time_cur &&
            c.endramp != 1) {
          end_ramp = true;
          c.endramp = 1;
        }
        enqueue_accept(c, end_ramp, c.st);
        c.time_cur = c.time_cur + h_loc[i];
        dt_correc = std::fabs(error) < TINY ? 2.0 : 0.9 * std::pow(error / P.toler, -(1.0 / 4.0));
      }
      double hr = h_rk[i] * dt_correc;
      hr = std::min(std::min(hr, 0.95 * P.dt_stab), P.delt_out);
      hr = std::max(std::max(hr, 0.0001 * 0.95 * P.dt_stab), 0.0001 * P.delt_out);
      h_rk[i] = hr;
      if (c.time_cur < time_next[i]) rc = launch(i);
      else --running;
    }
  }
  for (int i = 0; i < n; ++i) {
    Ctx& c = ctxs[i]->c;
    cudaStreamSynchronize(c.st);
    if (done[i]) cudaEventDestroy(done[i]);
    if (rc == HOSNWT_OK) rc = cuda_check(c, "advance_many");
  }
  return rc;
}

extern "C" int hosnwt_time_transform(hosnwt_ctx* h, int grid, int dir, int csx, int csy, int nin1,
                                     int nin2, int nout1, int nout2, int batch, int nrep,
                                     double* ms_per_launch) {
  if (!h || !ms_per_launch || batch < 1 || batch > kMaxJobs || nrep < 1) return HOSNWT_ERR_ARG;
  Ctx& c = h->c;
  const Params& P = c.P;
  int a = P.n1, b = P.n2;
  if (grid == GRID_BIG) { a = P.nd1; b = P.nd2; }
  else if (grid == GRID_ADD) { a = P.n3a; b = P.n2; }
  if (nin1 < 1 || nin1 > a || nout1 < 1 || nout1 > a || nin2 < 1 || nin2 > b || nout2 < 1 || nout2 > b)
    return HOSNWT_ERR_ARG;
  const size_t n = (size_t)a * b;
  std::vector<double*> bufs;
  for (int i = 0; i < 2 * batch; ++i) {
    double* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) {
      for (double* q : bufs) cudaFree(q);
      return fail(c, HOSNWT_ERR_CUDA, "time_transform: allocation failed");
    }
    std::vector<double> ones(n, 1.0);
    cudaMemcpy(p, ones.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    bufs.push_back(p);
  }
  std::vector<XfReq> rq(batch);
  for (int i = 0; i < batch; ++i) {
    XfReq& r = rq[i];
    r.grid = grid; r.dir = dir; r.csx = csx; r.csy = csy;
    r.in = bufs[2 * i]; r.in_ld = a; r.nin1 = nin1; r.nin2 = nin2;
    r.out = bufs[2 * i + 1]; r.out_ld = a; r.nout1 = nout1; r.nout2 = nout2;
    r.scale = 1.0;
  }
  // nrep back-to-back transforms captured in one graph, as the step graph
  // launches them; the second replay is timed
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // the first warm-up records the FFT batches for the layout tuner, as the
  // step graph's first capture does
  fft_tune_record(fft_tune_enabled());
  launch_transforms(rq.data(), batch, c.tb, c.d.xtmp, c.st);
  fft_tune_record(false);
  if (fft_tune_run(c.st) < 0) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (double* q : bufs) cudaFree(q);
    return fail(c, HOSNWT_ERR_CUDA, "time_transform: FFT layout tuning failed");
  }
  for (int w = 0; w < 2; ++w) launch_transforms(rq.data(), batch, c.tb, c.d.xtmp, c.st);
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  float ms = 0.f;
  bool ok = cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    for (int r = 0; r < nrep; ++r) launch_transforms(rq.data(), batch, c.tb, c.d.xtmp, c.st);
    ok = cudaStreamEndCapture(c.st, &g) == cudaSuccess;
  }
  if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
  if (ok) {
    cudaGraphLaunch(ge, c.st);
    cudaEventRecord(e0, c.st);
    cudaGraphLaunch(ge, c.st);
    cudaEventRecord(e1, c.st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
  }
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (double* q : bufs) cudaFree(q);
  if (!ok) return fail(c, HOSNWT_ERR_CUDA, "time_transform: graph capture failed");
  *ms_per_launch = ms / nrep;
  return cuda_check(c, "time_transform");
}

extern "C" int hosnwt_fp64_peak(double* gflops) {
  if (!gflops) return HOSNWT_ERR_ARG;
  *gflops = measure_fp64_peak_gflops();
  return *gflops > 0 ? HOSNWT_OK : HOSNWT_ERR_CUDA;
}
