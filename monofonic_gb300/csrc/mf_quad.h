// Adaptive Gauss-Kronrod quadrature (host): the integrator the reference's
// cosmology calculator uses for the sigma_8 normalisation
// (include/cosmology_calculator.hh:62-83: GSL's gsl_integration_qag with the
// 61-point rule, relative tolerance 1e-10).  Restated from the published
// algorithms, with the rule computed rather than tabulated:
//
//  * the n-point Gauss-Legendre nodes by Newton iteration on P_n;
//  * the n+1 Kronrod nodes as the zeros of the Stieltjes polynomial E_{n+1},
//    the polynomial of degree n+1 orthogonal to P_n x^k for k <= n -- here
//    expanded in Legendre polynomials and solved from those orthogonality
//    conditions (the integrals by exact Gauss quadrature), its zeros found by
//    bisection in the gaps between the Gauss nodes;
//  * the 2n+1 Kronrod weights from the moment equations
//    sum_i w_i P_m(x_i) = 2 delta_m0, m <= 2n;
//  all in long double.  The 61-point rule (n = 30) integrates polynomials of
//  degree 91 exactly;
//  * QAG (Piessens, de Doncker-Kapenga, Ueberhuber & Kahaner, QUADPACK,
//    1983): bisection of the interval with the largest error estimate until
//    the summed estimate is below max(epsabs, epsrel |I|), with QUADPACK's
//    error estimate of one rule application
//    err = resasc min(1, (200 |K - G| / resasc)^1.5), at least 50 eps resabs,
//    and its roundoff and interval-size termination tests.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <vector>

namespace mf {
namespace quad {

using ld = long double;

struct GKRule {
  int n = 0;               // Gauss points
  std::vector<double> xk;  // 2n+1 Kronrod nodes, ascending, symmetric
  std::vector<double> wk;  // Kronrod weights
  std::vector<double> wg;  // Gauss weights on the Kronrod grid (0 at Kronrod-only nodes)
};

// P_0..P_m at x (Bonnet's recursion)
inline void legendre_all(int m, ld x, std::vector<ld>& p) {
  p.assign(m + 1, 0.0L);
  p[0] = 1.0L;
  if (m >= 1) p[1] = x;
  for (int k = 1; k < m; ++k) p[k + 1] = ((2 * k + 1) * x * p[k] - k * p[k - 1]) / (k + 1);
}

inline void legendre_d(int n, ld x, ld& pn, ld& dpn) {
  ld p0 = 1.0L, p1 = x;
  for (int k = 1; k < n; ++k) {
    const ld p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
    p0 = p1;
    p1 = p2;
  }
  pn = p1;
  dpn = n * (x * p1 - p0) / (x * x - 1.0L);
}

// n-point Gauss-Legendre nodes (ascending) and weights on [-1, 1], n >= 2
inline void gauss_legendre(int n, std::vector<ld>& x, std::vector<ld>& w) {
  x.resize(n);
  w.resize(n);
  const ld pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < n; ++i) {
    ld z = std::cos(pi * (i + 0.75L) / (n + 0.5L));
    for (int it = 0; it < 100; ++it) {
      ld p, dp;
      legendre_d(n, z, p, dp);
      const ld dz = p / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-30L) break;
    }
    ld p, dp;
    legendre_d(n, z, p, dp);
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0L / ((1.0L - z * z) * dp * dp);
  }
}

// dense solve with partial pivoting; A row-major m x m, b overwritten by x
inline bool solve_dense(std::vector<ld> A, std::vector<ld>& b, int m) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int r = c + 1; r < m; ++r)
      if (std::fabs(A[(size_t)r * m + c]) > std::fabs(A[(size_t)piv * m + c])) piv = r;
    if (A[(size_t)piv * m + c] == 0.0L) return false;
    if (piv != c) {
      for (int k = 0; k < m; ++k) std::swap(A[(size_t)c * m + k], A[(size_t)piv * m + k]);
      std::swap(b[c], b[piv]);
    }
    for (int r = c + 1; r < m; ++r) {
      const ld f = A[(size_t)r * m + c] / A[(size_t)c * m + c];
      if (f == 0.0L) continue;
      for (int k = c; k < m; ++k) A[(size_t)r * m + k] -= f * A[(size_t)c * m + k];
      b[r] -= f * b[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    ld s = b[c];
    for (int k = c + 1; k < m; ++k) s -= A[(size_t)c * m + k] * b[k];
    b[c] = s / A[(size_t)c * m + c];
  }
  return true;
}

// the (2n+1)-point Gauss-Kronrod rule; an empty rule (n = 0) on failure
inline GKRule make_rule(int n) {
  GKRule R;
  std::vector<ld> xg, wg;
  gauss_legendre(n, xg, wg);
  const int Q = 2 * n + 8;  // exact for the degree-(3n+1) orthogonality integrands
  std::vector<ld> xq, wq;
  gauss_legendre(Q, xq, wq);
  std::vector<std::vector<ld>> Pq(Q);
  for (int q = 0; q < Q; ++q) legendre_all(n + 1, xq[q], Pq[q]);
  // E = P_{n+1} + sum_j c_j P_j over j of the parity of n+1; the conditions
  // int E P_n P_k = 0 that do not vanish by symmetry are those with k odd
  std::vector<int> js, ks;
  for (int j = (n + 1) % 2; j < n + 1; j += 2) js.push_back(j);
  for (int k = 1; k <= n; k += 2) ks.push_back(k);
  const int m = (int)js.size();
  if ((int)ks.size() != m) return GKRule{};
  std::vector<ld> A((size_t)m * m), b(m);
  for (int r = 0; r < m; ++r) {
    for (int c = 0; c < m; ++c) {
      ld s = 0.0L;
      for (int q = 0; q < Q; ++q) s += wq[q] * Pq[q][js[c]] * Pq[q][n] * Pq[q][ks[r]];
      A[(size_t)r * m + c] = s;
    }
    ld s = 0.0L;
    for (int q = 0; q < Q; ++q) s += wq[q] * Pq[q][n + 1] * Pq[q][n] * Pq[q][ks[r]];
    b[r] = -s;
  }
  if (!solve_dense(A, b, m)) return GKRule{};
  std::vector<ld> coef(n + 2, 0.0L);
  coef[n + 1] = 1.0L;
  for (int c = 0; c < m; ++c) coef[js[c]] = b[c];
  auto E = [&](ld x) {
    std::vector<ld> p;
    legendre_all(n + 1, x, p);
    ld s = 0.0L;
    for (int j = 0; j <= n + 1; ++j) s += coef[j] * p[j];
    return s;
  };
  std::vector<ld> xkro;
  for (int g = 0; g <= n; ++g) {
    ld lo = (g == 0) ? -1.0L : xg[g - 1];
    ld hi = (g == n) ? 1.0L : xg[g];
    ld flo = E(lo);
    if (flo * E(hi) > 0.0L) return GKRule{};
    for (int it = 0; it < 200; ++it) {
      const ld mid = 0.5L * (lo + hi);
      const ld fm = E(mid);
      if (fm == 0.0L) { lo = hi = mid; break; }
      if ((fm < 0.0L) == (flo < 0.0L)) { lo = mid; flo = fm; } else { hi = mid; }
    }
    xkro.push_back(0.5L * (lo + hi));
  }
  const int K = 2 * n + 1;
  std::vector<ld> xall;
  for (int i = 0; i < n; ++i) { xall.push_back(xkro[i]); xall.push_back(xg[i]); }
  xall.push_back(xkro[n]);
  for (int i = 0; i < K / 2; ++i) {  // the rule is symmetric about 0
    const ld v = 0.5L * (xall[K - 1 - i] - xall[i]);
    xall[i] = -v;
    xall[K - 1 - i] = v;
  }
  xall[K / 2] = 0.0L;
  std::vector<ld> M((size_t)K * K), rhs(K, 0.0L);
  for (int i = 0; i < K; ++i) {
    std::vector<ld> p;
    legendre_all(K - 1, xall[i], p);
    for (int mm = 0; mm < K; ++mm) M[(size_t)mm * K + i] = p[mm];
  }
  rhs[0] = 2.0L;
  if (!solve_dense(M, rhs, K)) return GKRule{};
  R.n = n;
  R.xk.resize(K);
  R.wk.resize(K);
  R.wg.assign(K, 0.0);
  for (int i = 0; i < K; ++i) {
    R.xk[i] = (double)xall[i];
    R.wk[i] = (double)(0.5L * (rhs[i] + rhs[K - 1 - i]));
  }
  for (int i = 0; i < n; ++i) R.wg[2 * i + 1] = (double)(0.5L * (wg[i] + wg[n - 1 - i]));
  return R;
}

// one rule application on [a, b]: integral, QUADPACK error estimate, and the
// integrals of |f| and |f - mean|
template <class F>
inline void qk(const GKRule& R, F& f, double a, double b, double* result, double* abserr, double* resabs,
               double* resasc) {
  const double center = 0.5 * (a + b), half = 0.5 * (b - a), ahalf = std::fabs(half);
  const int K = (int)R.xk.size();
  std::vector<double> fv(K);
  double rk = 0.0, rg = 0.0, ra = 0.0;
  for (int i = 0; i < K; ++i) {
    fv[i] = f(center + half * R.xk[i]);
    rk += R.wk[i] * fv[i];
    rg += R.wg[i] * fv[i];
    ra += R.wk[i] * std::fabs(fv[i]);
  }
  const double mean = 0.5 * rk;
  double rasc = 0.0;
  for (int i = 0; i < K; ++i) rasc += R.wk[i] * std::fabs(fv[i] - mean);
  *result = rk * half;
  *resabs = ra * ahalf;
  *resasc = rasc * ahalf;
  double err = std::fabs((rk - rg) * half);
  if (*resasc != 0.0 && err != 0.0) {
    const double scale = std::pow(200.0 * err / *resasc, 1.5);
    err = (scale < 1.0) ? *resasc * scale : *resasc;
  }
  if (*resabs > DBL_MIN / (50.0 * DBL_EPSILON)) {
    const double min_err = 50.0 * DBL_EPSILON * *resabs;
    if (min_err > err) err = min_err;
  }
  *abserr = err;
}

// QAG status: 0 converged, 1 roundoff on the first attempt, 2 iteration
// limit, 3 roundoff during subdivision, 4 interval too small, 5 bad rule
enum { kOk = 0, kRoundFirst = 1, kMaxIter = 2, kRound = 3, kSingular = 4, kBadRule = 5 };

template <class F>
inline int qag(const GKRule& R, F f, double a, double b, double epsabs, double epsrel, size_t limit,
               double* result, double* abserr) {
  if (R.n == 0) return kBadRule;
  struct Iv {
    double a, b, r, e;
  };
  double r0, e0, ra0, rc0;
  qk(R, f, a, b, &r0, &e0, &ra0, &rc0);
  *result = r0;
  *abserr = e0;
  double tol = std::max(epsabs, epsrel * std::fabs(r0));
  const double round_off = 50.0 * DBL_EPSILON * ra0;
  if (e0 <= round_off && e0 > tol) return kRoundFirst;
  if ((e0 <= tol && e0 != rc0) || e0 == 0.0) return kOk;
  if (limit <= 1) return kMaxIter;
  std::vector<Iv> iv{{a, b, r0, e0}};
  double area = r0, errsum = e0;
  int rt1 = 0, rt2 = 0, error_type = 0;
  size_t it = 1;
  do {
    size_t imax = 0;
    for (size_t i = 1; i < iv.size(); ++i)
      if (iv[i].e > iv[imax].e) imax = i;
    const Iv cur = iv[imax];
    const double a1 = cur.a, b1 = 0.5 * (cur.a + cur.b), a2 = b1, b2 = cur.b;
    double r1, e1, ra1, rc1, r2, e2, ra2, rc2;
    qk(R, f, a1, b1, &r1, &e1, &ra1, &rc1);
    qk(R, f, a2, b2, &r2, &e2, &ra2, &rc2);
    const double area12 = r1 + r2, error12 = e1 + e2;
    errsum += error12 - cur.e;
    area += area12 - cur.r;
    if (rc1 != e1 && rc2 != e2) {
      const double delta = cur.r - area12;
      if (std::fabs(delta) <= 1.0e-5 * std::fabs(area12) && error12 >= 0.99 * cur.e) ++rt1;
      if (it >= 10 && error12 > cur.e) ++rt2;
    }
    tol = std::max(epsabs, epsrel * std::fabs(area));
    if (errsum > tol) {
      if (rt1 >= 6 || rt2 >= 20) error_type = kRound;
      if (std::max(std::fabs(a1), std::fabs(b2)) <= (1.0 + 100.0 * DBL_EPSILON) * (std::fabs(a2) + 1000.0 * DBL_MIN))
        error_type = kSingular;
    }
    iv[imax] = {a1, b1, r1, e1};
    iv.push_back({a2, b2, r2, e2});
    ++it;
  } while (it < limit && !error_type && errsum > tol);
  double sum = 0.0;
  for (const Iv& v : iv) sum += v.r;
  *result = sum;
  *abserr = errsum;
  if (errsum <= tol) return kOk;
  return error_type ? error_type : kMaxIter;
}

}  // namespace quad
}  // namespace mf
