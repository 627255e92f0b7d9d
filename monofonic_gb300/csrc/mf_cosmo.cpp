// Host cosmology calculator and white-noise plugin.
//
// Restates, in this library's own code, the reference's host-side scalar
// producer: derived parameters (include/cosmology_parameters.hh:84-196),
// linear growth D+(a) from the single-fluid ODE with a Cash-Karp
// quality-controlled Runge-Kutta stepper (include/cosmology_calculator.hh:91-151,
// include/math/ode_integrate.hh:39-111), log-log natural cubic-spline
// interpolation of the tables (include/math/interpolate.hh:29-103), vfac
// (cosmology_calculator.hh:360-363) and the sigma_8 normalisation
// (cosmology_calculator.hh:368-380, 439-463).  The sigma_8 integral is the
// same QAG with the 61-point Gauss-Kronrod rule to relative 1e-10 (mf_quad.h,
// the rule computed rather than tabulated), so the scalars follow the
// reference's to rounding.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "../../include/monofonic_gb300_ic.h"
#include "mf_cosmo.h"
#include "mf_eh.cuh"
#include "mf_noise.h"
#include "mf_quad.h"

namespace mf {

// ---------------------------------------------------------------------------
// Eisenstein & Hu parameters (TFset_parameters, transfer_eisenstein.cc:58-122)
// ---------------------------------------------------------------------------
void eh_setup(double H0, double Omega_m, double Omega_b, double Tcmb, EHParams* p) {
  const double omhh = Omega_m * H0 * H0 * (0.01 * 0.01);
  const double f_baryon = Omega_b / Omega_m;
  p->m_h0 = H0 * 0.01;
  p->omhh = omhh;
  p->obhh = omhh * f_baryon;
  if (Tcmb <= 0.0) Tcmb = 2.728;
  const double th = Tcmb / 2.7, th2 = th * th, th4 = th2 * th2;
  const double z_equality = 2.50e4 * omhh / th4;
  p->k_equality = 0.0746 * omhh / th2;
  const double b1 = 0.313 * std::pow(omhh, -0.419) * (1 + 0.607 * std::pow(omhh, 0.674));
  const double b2 = 0.238 * std::pow(omhh, 0.223);
  const double z_drag = 1291 * std::pow(omhh, 0.251) / (1 + 0.659 * std::pow(omhh, 0.828)) *
                        (1 + b1 * std::pow(p->obhh, b2));
  const double R_drag = 31.5 * p->obhh / th4 * (1000 / (1 + z_drag));
  const double R_eq = 31.5 * p->obhh / th4 * (1000 / z_equality);
  p->sound_horizon = 2. / 3. / p->k_equality * std::sqrt(6. / R_eq) *
                     std::log((std::sqrt(1 + R_drag) + std::sqrt(R_drag + R_eq)) / (1 + std::sqrt(R_eq)));
  p->k_silk = 1.6 * std::pow(p->obhh, 0.52) * std::pow(omhh, 0.73) * (1 + std::pow(10.4 * omhh, -0.95));
  const double a1 = std::pow(46.9 * omhh, 0.670) * (1 + std::pow(32.1 * omhh, -0.532));
  const double a2 = std::pow(12.0 * omhh, 0.424) * (1 + std::pow(45.0 * omhh, -0.582));
  p->alpha_c = std::pow(a1, -f_baryon) * std::pow(a2, -(f_baryon * f_baryon * f_baryon));
  const double bb1 = 0.944 / (1 + std::pow(458 * omhh, -0.708));
  const double bb2 = std::pow(0.395 * omhh, -0.0266);
  p->beta_c = 1.0 / (1 + bb1 * (std::pow(1 - f_baryon, bb2) - 1));
  const double y = z_equality / (1 + z_drag);
  const double G = y * (-6. * std::sqrt(1 + y) + (2. + 3. * y) * std::log((std::sqrt(1 + y) + 1) / (std::sqrt(1 + y) - 1)));
  p->alpha_b = 2.07 * p->k_equality * p->sound_horizon * std::pow(1 + R_drag, -0.75) * G;
  p->beta_node = 8.41 * std::pow(omhh, 0.435);
  p->beta_b = 0.5 + f_baryon + (3. - 2. * f_baryon) * std::sqrt(std::pow(17.2 * omhh, 2.0) + 1);
  p->fb = Omega_b / Omega_m;
  p->fc = (Omega_m - Omega_b) / Omega_m;
}

double eh_at_k(const EHParams& p, double k) { return eh_eval(p, k); }

namespace {

// physical constants (include/physical_constants.hh:24-63)
constexpr double kPi = 3.141592653589793115997963468544185161590576171875;
constexpr double kMpc = 3.0857e22, kC = 2.99792458e8, kG = 6.6740800e-11, kKB = 1.38064852e-23,
                 kHbar = 1.054571800e-34;
const double kSigmaSB = (kPi * kPi) * (kKB * kKB * kKB * kKB) / 60. / (kHbar * kHbar * kHbar) / (kC * kC);
const double kRhoCrit = 3 * 1e10 / (8 * kPi * kG) / kMpc / kMpc;

struct Cosmo {
  double h, H0, Omega_m, Omega_b, Omega_r, Omega_DE, Omega_k, w0, wa, n_s, sigma8, Tcmb;
  double H(double a) const {
    const double HH2 = Omega_r / (a * a * a * a) + Omega_m / (a * a * a) + Omega_k / (a * a) +
                       Omega_DE * std::pow(a, -3. * (1. + w0 + wa)) * std::exp(-3. * (1.0 - a) * wa);
    return H0 * std::sqrt(HH2);
  }
};

Cosmo derive(const mf_cosmo_params& in) {
  Cosmo c{};
  c.h = in.h;
  c.H0 = 100.0 * in.h;
  c.Omega_m = in.Omega_m;
  c.Omega_b = in.Omega_b;
  c.n_s = in.n_s;
  c.sigma8 = in.sigma_8;
  c.w0 = in.w_0;
  c.wa = in.w_a;
  c.Tcmb = in.Tcmb > 0 ? in.Tcmb : 2.7255;
  const double m_nu1 = in.m_nu1 >= 0 ? in.m_nu1 : 0.06;
  const int n_massive = (m_nu1 > 1e-9) ? 1 : 0;
  const double N_ur = in.N_ur >= 0 ? in.N_ur : 3.046 - n_massive;
  const double Omega_gamma = 4 * kSigmaSB / (kC * kC * kC) * std::pow(c.Tcmb, 4.0) / kRhoCrit / (c.h * c.h);
  const double Omega_nu = N_ur * Omega_gamma * 7. / 8. * std::pow(4. / 11., 4. / 3.);
  c.Omega_r = in.zero_radiation ? 0.0 : Omega_gamma + Omega_nu;
  double ODE = in.Omega_L >= 0 ? in.Omega_L : 0.6901;
  ODE += 1.0 - c.Omega_m - ODE - c.Omega_r;  // flat closure (cosmology_parameters.hh:170-173)
  c.Omega_DE = ODE;
  c.Omega_k = 0.0;
  return c;
}

using V3 = std::array<double, 3>;

// growth tables (a, D, f), compute_growth (cosmology_calculator.hh:91-151)
void growth_tables(const Cosmo& c, std::vector<double>& ta, std::vector<double>& tD, std::vector<double>& tf) {
  constexpr double a2 = 0.20, a3 = 0.30, a4 = 0.60, a5 = 1.0, a6 = 0.8750;
  constexpr double b21 = 0.20, b31 = 3.0 / 40.0, b32 = 9.0 / 40.0, b41 = 0.30, b42 = -0.90, b43 = 1.20,
                   b51 = -11.0 / 54.0, b52 = 2.50, b53 = -70.0 / 27.0, b54 = 35.0 / 27.0, b61 = 1631.0 / 55296.0,
                   b62 = 175.0 / 512.0, b63 = 575.0 / 13824.0, b64 = 44275.0 / 110592.0, b65 = 253.0 / 4096.0,
                   c1 = 37.0 / 378.0, c3 = 250.0 / 621.0, c4 = 125.0 / 594.0, c6 = 512.0 / 1771.0;
  constexpr double dc1 = c1 - 2825.0 / 27648.0, dc3 = c3 - 18575.0 / 48384.0, dc4 = c4 - 13525.0 / 55296.0,
                   dc5 = -277.0 / 14336.0, dc6 = c6 - 0.250;
  (void)a2; (void)a3; (void)a4; (void)a5; (void)a6;  // autonomous system: stage times unused
  const double Om = c.Omega_m, H0 = c.H0;
  auto rhs = [&](const V3& y) -> V3 {
    const double a = y[0], D = y[1], Dp = y[2];
    const double Ha = c.H(a);
    return V3{a * a * Ha, Dp, -a * Ha * Dp + 3.0 / 2.0 * Om * H0 * H0 * D / a};
  };
  auto axpy = [](const V3& y, std::initializer_list<std::pair<double, const V3*>> terms) {
    V3 r = y;
    for (auto& t : terms)
      for (int i = 0; i < 3; ++i) r[i] += t.first * (*t.second)[i];
    return r;
  };
  const double a0 = 1e-10;
  V3 y{a0, a0, 2.0 * a0 * c.H(a0) / (kC * kC)};
  double dt = 1e-9;
  const double eps = 1e-10;
  while (y[0] < 2.0) {
    const V3 f0 = rhs(y);
    V3 yscale;
    for (int i = 0; i < 3; ++i) yscale[i] = std::fabs(y[i]) + dt * std::fabs(f0[i]);
    double h = dt, hnext = dt;
    // the trial state: each trial advances it in place, and a rejected trial
    // is retried from the state it left behind, as the reference's
    // rk_step_qs does (ckrk5_step updates ytemp, which is not reset before
    // the retry; include/math/ode_integrate.hh:73-110)
    V3 yt = y;
    for (;;) {
      const V3 base = yt;
      V3 k1 = rhs(base); for (auto& v : k1) v *= h;
      V3 k2 = rhs(axpy(base, {{b21, &k1}})); for (auto& v : k2) v *= h;
      V3 k3 = rhs(axpy(base, {{b31, &k1}, {b32, &k2}})); for (auto& v : k3) v *= h;
      V3 k4 = rhs(axpy(base, {{b41, &k1}, {b42, &k2}, {b43, &k3}})); for (auto& v : k4) v *= h;
      V3 k5 = rhs(axpy(base, {{b51, &k1}, {b52, &k2}, {b53, &k3}, {b54, &k4}})); for (auto& v : k5) v *= h;
      V3 k6 = rhs(axpy(base, {{b61, &k1}, {b62, &k2}, {b63, &k3}, {b64, &k4}, {b65, &k5}})); for (auto& v : k6) v *= h;
      yt = axpy(base, {{c1, &k1}, {c3, &k3}, {c4, &k4}, {c6, &k6}});
      double errmax = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double e = dc1 * k1[i] + dc3 * k3[i] + dc4 * k4[i] + dc5 * k5[i] + dc6 * k6[i];
        errmax = std::max(errmax, std::fabs(e / yscale[i]));
      }
      errmax /= eps;
      if (errmax > 1.0) {
        h *= std::max(0.1, 0.9 * std::pow(errmax, -0.25));
        continue;
      }
      hnext = (errmax > 1.89e-4) ? h * 0.9 * std::pow(errmax, -0.2) : 5 * h;
      y = yt;
      break;
    }
    ta.push_back(y[0]);
    tD.push_back(y[1]);
    tf.push_back(y[2]);
    dt = hnext;
  }
  for (size_t i = 0; i < ta.size(); ++i) tf[i] = tf[i] / (ta[i] * c.H(ta[i]) * tD[i]);
}

// natural cubic spline of log y against log x
class LogLogSpline {
 public:
  LogLogSpline(const std::vector<double>& x, const std::vector<double>& y) {
    const size_t n = x.size();
    x_.resize(n); y_.resize(n); m_.assign(n, 0.0);
    for (size_t i = 0; i < n; ++i) { x_[i] = std::log(x[i]); y_[i] = std::log(y[i]); }
    // tridiagonal system for the second derivatives, natural end conditions
    std::vector<double> cp(n, 0.0), dp(n, 0.0);
    for (size_t i = 1; i + 1 < n; ++i) {
      const double h0 = x_[i] - x_[i - 1], h1 = x_[i + 1] - x_[i];
      const double a = h0 / 6.0, b = (h0 + h1) / 3.0, cc = h1 / 6.0;
      const double d = (y_[i + 1] - y_[i]) / h1 - (y_[i] - y_[i - 1]) / h0;
      const double den = b - a * cp[i - 1];
      cp[i] = cc / den;
      dp[i] = (d - a * dp[i - 1]) / den;
    }
    for (size_t i = n - 2; i >= 1; --i) {
      m_[i] = dp[i] - cp[i] * m_[i + 1];
      if (i == 1) break;
    }
  }
  double operator()(double xv) const {
    const double x = std::log(xv);
    size_t hi = std::upper_bound(x_.begin(), x_.end(), x) - x_.begin();
    if (hi == 0) hi = 1;
    if (hi >= x_.size()) hi = x_.size() - 1;
    const size_t lo = hi - 1;
    const double h = x_[hi] - x_[lo];
    const double A = (x_[hi] - x) / h, B = (x - x_[lo]) / h;
    const double y = A * y_[lo] + B * y_[hi] + ((A * A * A - A) * m_[lo] + (B * B * B - B) * m_[hi]) * h * h / 6.0;
    return std::exp(y);
  }

 private:
  std::vector<double> x_, y_, m_;
};

}  // namespace
}  // namespace mf

using namespace mf;

extern "C" void mf_cosmo_params_default(mf_cosmo_params* p) {
  if (!p) return;
  p->Omega_m = 0.3099;
  p->Omega_b = 0.048891054;
  p->h = 0.67742;
  p->sigma_8 = 0.8102;
  p->n_s = 0.96822;
  p->Omega_L = -1.0;
  p->Tcmb = -1.0;
  p->m_nu1 = -1.0;
  p->N_ur = -1.0;
  p->w_0 = -1.0;
  p->w_a = 0.0;
  p->zero_radiation = 0;
}

extern "C" int mf_cosmology_compute(const mf_cosmo_params* p, double zstart, mf_cosmo_scalars* out) {
  if (!p || !out) return MF_ERR_ARG;
  if (!(p->Omega_m > 0) || !(p->Omega_b > 0) || !(p->h > 0) || !(p->sigma_8 > 0) || !(zstart >= 0))
    return MF_ERR_ARG;
  const Cosmo c = derive(*p);
  std::vector<double> ta, tD, tf;
  growth_tables(c, ta, tD, tf);
  if (ta.size() < 6) return MF_ERR_ARG;
  LogLogSpline D_of_a(ta, tD), f_of_a(ta, tf);
  const double Dnow = D_of_a(1.0);
  const double astart = 1.0 / (1.0 + zstart);
  out->Dplus = D_of_a(astart) / Dnow;
  out->f = f_of_a(astart);
  out->vfac = out->f * astart * c.H(astart) / c.h;
  EHParams eh;
  eh_setup(c.H0, c.Omega_m, c.Omega_b, c.Tcmb, &eh);
  const double ns = c.n_s;
  auto dsig = [&](double k) {
    const double x = k * 8.0;
    const double w = (x < 0.001) ? 1.0 - 0.1 * x * x : 3.0 * (std::sin(x) - x * std::cos(x)) / (x * x * x);
    const double tk = eh_eval(eh, k);
    return k * k * w * w * std::pow(k, ns) * tk * tk;
  };
  // the reference's integrate(): QAG with the 61-point Gauss-Kronrod rule to
  // relative 1e-10 over the transfer plugin's [kmin, kmax] = [1e-4, 1e4]
  // (cosmology_calculator.hh:62-83, 439-452; transfer_eisenstein.cc:243-251)
  static const quad::GKRule gk61 = quad::make_rule(30);
  double sig_int = 0.0, sig_err = 0.0;
  quad::qag(gk61, dsig, 1e-4, 1e4, 0.0, 1e-10, 100000, &sig_int, &sig_err);
  const double sigma0 = 4.0 * M_PI * sig_int;
  out->sigma8_measured = std::sqrt(sigma0);
  out->pnorm = c.sigma8 * c.sigma8 / (out->sigma8_measured * out->sigma8_measured);
  out->n_s = ns;
  out->h = c.h;
  out->H0 = c.H0;
  out->Omega_m = c.Omega_m;
  out->Omega_b = c.Omega_b;
  out->Omega_r = c.Omega_r;
  out->Omega_DE = c.Omega_DE;
  out->Tcmb = c.Tcmb;
  return MF_OK;
}

extern "C" int mf_eh_transfer(const mf_cosmo_params* p, const double* k, double* out, size_t n) {
  if (!p || (n && (!k || !out))) return MF_ERR_ARG;
  const Cosmo c = derive(*p);
  EHParams eh;
  eh_setup(c.H0, c.Omega_m, c.Omega_b, c.Tcmb, &eh);
  for (size_t i = 0; i < n; ++i) out[i] = eh_eval(eh, k[i]);
  return MF_OK;
}

extern "C" int mf_white_noise_host(int n, uint64_t seed, double* out, int nthreads) {
  if (n <= 0 || !out) return MF_ERR_ARG;
  const uint64_t ncell = (uint64_t)n * n * n, npair = (ncell + 1) / 2;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  auto work = [&](uint64_t p0, uint64_t p1) {
    for (uint64_t p = p0; p < p1; ++p) {
      double z0, z1;
      noise::normal_pair(p, seed, &z0, &z1);
      out[2 * p] = z0;
      if (2 * p + 1 < ncell) out[2 * p + 1] = z1;
    }
  };
  std::vector<std::thread> th;
  const uint64_t chunk = (npair + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    const uint64_t p0 = t * chunk, p1 = std::min(npair, p0 + chunk);
    if (p0 >= p1) break;
    th.emplace_back(work, p0, p1);
  }
  for (auto& t : th) t.join();
  return MF_OK;
}
