// Project implementations behind the GSL-API shim headers (gsl/*.h).  Test
// infrastructure for oracle/_ref only: they let the reference's cosmology
// calculator, splines and PLT eigen-decompositions run unmodified without GSL.
//
//  * gsl_integration_qag: the project's QUADPACK QAG on computed
//    Gauss-Kronrod rules (monofonic_gb300/csrc/mf_quad.h, the same routine
//    the pipeline's host cosmology uses); GSL_INTEG_GAUSS61 is n = 30.
//  * gsl_spline (cspline): the natural cubic spline, y'' = 0 at both ends,
//    second derivatives from the tridiagonal system (Thomas algorithm).
//  * gsl_eigen_symmv: cyclic Jacobi rotations (Jacobi 1846; Golub & Van Loan
//    section 8.5) to machine precision; eigenvectors orthonormal, their signs
//    as the rotations leave them (the reference aligns them with k).
//  * gsl_sf_hyperg_2F1: the hypergeometric series for |x| < 1.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <vector>

#include "gsl/gsl_eigen.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_sf_hyperg.h"
#include "gsl/gsl_spline.h"
#include "mf_quad.h"

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------
namespace {
void default_handler(const char* reason, const char* file, int line, int gsl_errno) {
  std::fprintf(stderr, "gsl shim: %s:%d: ERROR: %s (code %d)\n", file, line, reason, gsl_errno);
  std::abort();
}
void off_handler(const char*, const char*, int, int) {}
gsl_error_handler_t* g_handler = nullptr;  // nullptr: default (abort)
}  // namespace

extern "C" gsl_error_handler_t* gsl_set_error_handler(gsl_error_handler_t* h) {
  gsl_error_handler_t* old = g_handler;
  g_handler = h;
  return old;
}
extern "C" gsl_error_handler_t* gsl_set_error_handler_off(void) {
  gsl_error_handler_t* old = g_handler;
  g_handler = off_handler;
  return old;
}
extern "C" void gsl_error(const char* reason, const char* file, int line, int gsl_errno) {
  (g_handler ? g_handler : default_handler)(reason, file, line, gsl_errno);
}

// ---------------------------------------------------------------------------
// adaptive Gauss-Kronrod quadrature: the project's QAG (mf_quad.h)
// ---------------------------------------------------------------------------
namespace {
const mf::quad::GKRule& rule(int key) {
  static std::mutex mu;
  static mf::quad::GKRule rules[7];
  static const int npts[7] = {0, 7, 10, 15, 20, 25, 30};
  std::lock_guard<std::mutex> g(mu);
  if (key < 1 || key > 6) key = 6;
  if (rules[key].n == 0) rules[key] = mf::quad::make_rule(npts[key]);
  return rules[key];
}
}  // namespace

struct gsl_integration_workspace {
  size_t limit;
};

extern "C" gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) {
  return new gsl_integration_workspace{n};
}
extern "C" void gsl_integration_workspace_free(gsl_integration_workspace* w) { delete w; }

extern "C" int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs, double epsrel,
                                   size_t limit, int key, gsl_integration_workspace* ws, double* result,
                                   double* abserr) {
  if (ws && limit > ws->limit) limit = ws->limit;
  auto fn = [f](double x) { return f->function(x, f->params); };
  const int st = mf::quad::qag(rule(key), fn, a, b, epsabs, epsrel, limit, result, abserr);
  switch (st) {
    case mf::quad::kOk: return GSL_SUCCESS;
    case mf::quad::kRoundFirst:
      gsl_error("cannot reach tolerance because of roundoff error on first attempt", __FILE__, __LINE__, GSL_EROUND);
      return GSL_EROUND;
    case mf::quad::kRound:
      gsl_error("roundoff error prevents tolerance from being achieved", __FILE__, __LINE__, GSL_EROUND);
      return GSL_EROUND;
    case mf::quad::kSingular:
      gsl_error("bad integrand behavior found in the integration interval", __FILE__, __LINE__, GSL_ESING);
      return GSL_ESING;
    case mf::quad::kMaxIter:
      gsl_error("number of iterations was insufficient", __FILE__, __LINE__, GSL_EMAXITER);
      return GSL_EMAXITER;
    default:
      gsl_error("could not construct the Gauss-Kronrod rule", __FILE__, __LINE__, GSL_FAILURE);
      return GSL_FAILURE;
  }
}

// ---------------------------------------------------------------------------
// natural cubic spline
// ---------------------------------------------------------------------------
namespace {
const gsl_interp_type k_cspline = {"cspline", 0};
const gsl_interp_type k_cspline_periodic = {"cspline-periodic", 1};
}  // namespace
extern "C" {
const gsl_interp_type* gsl_interp_cspline = &k_cspline;
const gsl_interp_type* gsl_interp_cspline_periodic = &k_cspline_periodic;
}

struct gsl_spline {
  const gsl_interp_type* type;
  std::vector<double> x, y, c;  // c = y''/2 at the knots
};

extern "C" gsl_interp_accel* gsl_interp_accel_alloc(void) { return new gsl_interp_accel{0}; }
extern "C" void gsl_interp_accel_free(gsl_interp_accel* a) { delete a; }

extern "C" gsl_spline* gsl_spline_alloc(const gsl_interp_type* T, size_t size) {
  if (size < 3) {
    gsl_error("insufficient number of points for interpolation type", __FILE__, __LINE__, GSL_EINVAL);
    return nullptr;
  }
  gsl_spline* s = new gsl_spline;
  s->type = T;
  s->x.resize(size);
  s->y.resize(size);
  s->c.assign(size, 0.0);
  return s;
}

extern "C" int gsl_spline_init(gsl_spline* s, const double xa[], const double ya[], size_t size) {
  if (s->type->periodic) {
    gsl_error("periodic cubic splines are not provided by this shim", __FILE__, __LINE__, GSL_EINVAL);
    return GSL_EINVAL;
  }
  for (size_t i = 1; i < size; ++i)
    if (!(xa[i] > xa[i - 1])) {
      gsl_error("x values must be strictly increasing", __FILE__, __LINE__, GSL_EINVAL);
      return GSL_EINVAL;
    }
  s->x.assign(xa, xa + size);
  s->y.assign(ya, ya + size);
  const size_t n = size;
  // interior unknowns c_1..c_{n-2} (c = y''/2), c_0 = c_{n-1} = 0:
  // h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1} = 3 (s_i - s_{i-1})
  const size_t m = n - 2;
  std::vector<double> diag(m), off(m), rhs(m);
  for (size_t k = 0; k < m; ++k) {
    const size_t i = k + 1;
    const double h0 = xa[i] - xa[i - 1], h1 = xa[i + 1] - xa[i];
    diag[k] = 2.0 * (h0 + h1);
    off[k] = h1;
    rhs[k] = 3.0 * ((ya[i + 1] - ya[i]) / h1 - (ya[i] - ya[i - 1]) / h0);
  }
  // Thomas algorithm on the symmetric tridiagonal system
  for (size_t k = 1; k < m; ++k) {
    const double w = off[k - 1] / diag[k - 1];
    diag[k] -= w * off[k - 1];
    rhs[k] -= w * rhs[k - 1];
  }
  s->c.assign(n, 0.0);
  if (m > 0) {
    s->c[m] = rhs[m - 1] / diag[m - 1];
    for (size_t k = m - 1; k-- > 0;) s->c[k + 1] = (rhs[k] - off[k] * s->c[k + 2]) / diag[k];
  }
  return GSL_SUCCESS;
}

extern "C" double gsl_spline_eval(const gsl_spline* s, double x, gsl_interp_accel* a) {
  const size_t n = s->x.size();
  if (x < s->x[0] || x > s->x[n - 1]) {
    gsl_error("interpolation error", __FILE__, __LINE__, GSL_EDOM);
    return NAN;
  }
  size_t i;
  if (a && a->cache + 1 < n && s->x[a->cache] <= x && x <= s->x[a->cache + 1]) {
    i = a->cache;
  } else {
    i = (size_t)(std::upper_bound(s->x.begin(), s->x.end(), x) - s->x.begin());
    i = (i == 0) ? 0 : i - 1;
    if (i >= n - 1) i = n - 2;
    if (a) a->cache = i;
  }
  const double h = s->x[i + 1] - s->x[i], dx = x - s->x[i];
  const double ci = s->c[i], ci1 = s->c[i + 1];
  const double b = (s->y[i + 1] - s->y[i]) / h - h * (ci1 + 2.0 * ci) / 3.0;
  const double d = (ci1 - ci) / (3.0 * h);
  return s->y[i] + dx * (b + dx * (ci + dx * d));
}

extern "C" void gsl_spline_free(gsl_spline* s) { delete s; }

// ---------------------------------------------------------------------------
// matrices, vectors and the symmetric eigenproblem
// ---------------------------------------------------------------------------
extern "C" gsl_matrix_view gsl_matrix_view_array(double* base, size_t n1, size_t n2) {
  gsl_matrix_view v;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = n2;
  v.matrix.data = base;
  v.matrix.block = nullptr;
  v.matrix.owner = 0;
  return v;
}
extern "C" gsl_vector* gsl_vector_alloc(size_t n) {
  gsl_vector* v = new gsl_vector;
  v->size = n;
  v->stride = 1;
  v->data = new double[n]();
  v->block = nullptr;
  v->owner = 1;
  return v;
}
extern "C" void gsl_vector_free(gsl_vector* v) {
  if (!v) return;
  if (v->owner) delete[] v->data;
  delete v;
}
extern "C" gsl_matrix* gsl_matrix_alloc(size_t n1, size_t n2) {
  gsl_matrix* m = new gsl_matrix;
  m->size1 = n1;
  m->size2 = n2;
  m->tda = n2;
  m->data = new double[n1 * n2]();
  m->block = nullptr;
  m->owner = 1;
  return m;
}
extern "C" void gsl_matrix_free(gsl_matrix* m) {
  if (!m) return;
  if (m->owner) delete[] m->data;
  delete m;
}
extern "C" double gsl_vector_get(const gsl_vector* v, size_t i) { return v->data[i * v->stride]; }
extern "C" double gsl_matrix_get(const gsl_matrix* m, size_t i, size_t j) { return m->data[i * m->tda + j]; }

struct gsl_eigen_symmv_workspace {
  size_t n;
};
extern "C" gsl_eigen_symmv_workspace* gsl_eigen_symmv_alloc(size_t n) { return new gsl_eigen_symmv_workspace{n}; }
extern "C" void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace* w) { delete w; }

extern "C" int gsl_eigen_symmv(gsl_matrix* A, gsl_vector* eval, gsl_matrix* evec, gsl_eigen_symmv_workspace*) {
  const size_t n = A->size1;
  std::vector<double> a(n * n), v(n * n, 0.0);
  // symmetric input: the lower triangle and the diagonal are read, as GSL does
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) a[i * n + j] = a[j * n + i] = A->data[i * A->tda + j];
  for (size_t i = 0; i < n; ++i) v[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double offn = 0.0, diagn = 0.0;
    for (size_t i = 0; i < n; ++i) {
      diagn += a[i * n + i] * a[i * n + i];
      for (size_t j = i + 1; j < n; ++j) offn += a[i * n + j] * a[i * n + j];
    }
    if (offn == 0.0 || offn <= 1e-36 * diagn) break;
    for (size_t p = 0; p < n; ++p)
      for (size_t q = p + 1; q < n; ++q) {
        const double apq = a[p * n + q];
        if (apq == 0.0) continue;
        const double app = a[p * n + p], aqq = a[q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (size_t k = 0; k < n; ++k) {
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (size_t k = 0; k < n; ++k) {
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (size_t k = 0; k < n; ++k) {
          const double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (size_t i = 0; i < n; ++i) {
    eval->data[i * eval->stride] = a[i * n + i];
    for (size_t k = 0; k < n; ++k) evec->data[k * evec->tda + i] = v[k * n + i];
  }
  // the input matrix is used as workspace, as GSL does
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) A->data[i * A->tda + j] = a[i * n + j];
  return GSL_SUCCESS;
}

extern "C" int gsl_eigen_symmv_sort(gsl_vector* eval, gsl_matrix* evec, gsl_eigen_sort_t sort_type) {
  const size_t n = eval->size;
  for (size_t i = 0; i + 1 < n; ++i) {
    size_t k = i;
    double ek = eval->data[i * eval->stride];
    for (size_t j = i + 1; j < n; ++j) {
      const double ej = eval->data[j * eval->stride];
      bool better = false;
      switch (sort_type) {
        case GSL_EIGEN_SORT_VAL_ASC: better = ej < ek; break;
        case GSL_EIGEN_SORT_VAL_DESC: better = ej > ek; break;
        case GSL_EIGEN_SORT_ABS_ASC: better = std::fabs(ej) < std::fabs(ek); break;
        case GSL_EIGEN_SORT_ABS_DESC: better = std::fabs(ej) > std::fabs(ek); break;
      }
      if (better) { k = j; ek = ej; }
    }
    if (k != i) {
      std::swap(eval->data[i * eval->stride], eval->data[k * eval->stride]);
      for (size_t r = 0; r < n; ++r) std::swap(evec->data[r * evec->tda + i], evec->data[r * evec->tda + k]);
    }
  }
  return GSL_SUCCESS;
}

// ---------------------------------------------------------------------------
// 2F1(a, b; c; x) = sum_k (a)_k (b)_k / ((c)_k k!) x^k, |x| < 1
// ---------------------------------------------------------------------------
extern "C" double gsl_sf_hyperg_2F1(double a, double b, double c, double x) {
  if (!(std::fabs(x) < 1.0)) {
    gsl_error("2F1 series needs |x| < 1 in this shim", __FILE__, __LINE__, GSL_EDOM);
    return NAN;
  }
  double term = 1.0, sum = 1.0;
  for (int k = 0; k < 100000; ++k) {
    term *= (a + k) * (b + k) / ((c + k) * (k + 1.0)) * x;
    sum += term;
    if (std::fabs(term) < 1e-17 * std::fabs(sum)) break;
  }
  return sum;
}
