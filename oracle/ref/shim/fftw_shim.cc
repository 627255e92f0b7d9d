// Project CPU transform behind the FFTW3-API shim (fftw3.h).  Test
// infrastructure for oracle/_ref only: it lets the reference's own Grid_FFT
// (src/grid_fft.cc:40-270) run unmodified without FFTW.
//
// Line transforms: recursive decimation in time over the factors 4, 2, 3, 5
// and any remaining primes (direct DFT), twiddles exp(-2 pi i j / n) from a
// long-double table per length.  B = 8 lines are transformed together with
// their elements interleaved ([element][line]), so every butterfly runs over
// eight independent lines (contiguous rows and strided columns alike are
// gathered into that layout).
//
// 3D transforms follow FFTW's definitions:
//   r2c  X[k0,k1,k2] = sum_x x e^{-2 pi i k.x / n}, kz in [0, n2/2]; the
//        rows along n2 first (half-length complex transform of the packed
//        pairs), then the columns along n1 and n0;
//   c2r  the columns along n0 and n1 first (complex, sign +), then each row
//        along n2 as the inverse real transform of the Hermitian extension of
//        X[0..n2/2], reading only the real parts of the kz = 0 and kz = n2/2
//        terms -- the result FFTW's c2r gives for input that is not Hermitian
//        on those planes;
//   c2c  rows, then columns, sign as given; all unnormalised.
// In-place r2c/c2r arrays have rows of 2 (n2/2 + 1) reals, as FFTW's.
#include "fftw3.h"

#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <vector>

namespace {

struct cd {
  double re, im;
};
inline cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cd cconj(cd a) { return {a.re, -a.im}; }

constexpr int B = 8;
int g_threads = 0;  // 0: OpenMP's default

int nthreads() { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

struct LinePlan {
  int n = 0;
  std::vector<int> fac;
  std::vector<cd> w;  // w[j] = exp(-2 pi i j / n)
};

std::vector<int> factorize(int n) {
  std::vector<int> f;
  while (n % 4 == 0) { f.push_back(4); n /= 4; }
  while (n % 2 == 0) { f.push_back(2); n /= 2; }
  while (n % 3 == 0) { f.push_back(3); n /= 3; }
  while (n % 5 == 0) { f.push_back(5); n /= 5; }
  for (int p = 7; n > 1; p += 2)
    while (n % p == 0) { f.push_back(p); n /= p; }
  return f;
}

const LinePlan& line_plan(int n) {
  static std::mutex mu;
  static std::map<int, LinePlan*> cache;
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(n);
  if (it != cache.end()) return *it->second;
  LinePlan* p = new LinePlan;
  p->n = n;
  p->fac = factorize(n);
  p->w.resize(n);
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (int j = 0; j < n; ++j) {
    const long double a = -twopi * (long double)j / (long double)n;
    p->w[j] = {(double)cosl(a), (double)sinl(a)};
  }
  cache[n] = p;
  return *p;
}

inline cd twiddle(const LinePlan& P, int j, bool inv) {
  const cd w = P.w[j];
  return inv ? cconj(w) : w;
}

// y[p] = sum_q t[q] w_r^{pq} over B lines; t and y hold r B-vectors
void dft_small(const cd* t, cd* y, size_t ystride, int r, const LinePlan& P, bool inv) {
  if (r == 2) {
    for (int b = 0; b < B; ++b) {
      const cd a = t[b], c = t[B + b];
      y[b] = {a.re + c.re, a.im + c.im};
      y[ystride + b] = {a.re - c.re, a.im - c.im};
    }
    return;
  }
  if (r == 4) {
    for (int b = 0; b < B; ++b) {
      const cd a0 = t[b], a1 = t[B + b], a2 = t[2 * B + b], a3 = t[3 * B + b];
      const cd s0 = {a0.re + a2.re, a0.im + a2.im}, d0 = {a0.re - a2.re, a0.im - a2.im};
      const cd s1 = {a1.re + a3.re, a1.im + a3.im}, d1 = {a1.re - a3.re, a1.im - a3.im};
      // w_4 = -i forward, +i inverse: d1 * w_4
      const cd d1w = inv ? cd{-d1.im, d1.re} : cd{d1.im, -d1.re};
      y[b] = {s0.re + s1.re, s0.im + s1.im};
      y[2 * ystride + b] = {s0.re - s1.re, s0.im - s1.im};
      y[ystride + b] = {d0.re + d1w.re, d0.im + d1w.im};
      y[3 * ystride + b] = {d0.re - d1w.re, d0.im - d1w.im};
    }
    return;
  }
  if (r == 3) {
    const cd w1 = twiddle(P, P.n / 3, inv);  // exp(-+2 pi i / 3)
    for (int b = 0; b < B; ++b) {
      const cd a0 = t[b], a1 = t[B + b], a2 = t[2 * B + b];
      const cd s = {a1.re + a2.re, a1.im + a2.im}, d = {a1.re - a2.re, a1.im - a2.im};
      const cd m = {a0.re + w1.re * s.re, a0.im + w1.re * s.im};  // w1.re = -1/2
      // i * w1.im * d
      const cd r1 = {-w1.im * d.im, w1.im * d.re};
      y[b] = {a0.re + s.re, a0.im + s.im};
      y[ystride + b] = {m.re + r1.re, m.im + r1.im};
      y[2 * ystride + b] = {m.re - r1.re, m.im - r1.im};
    }
    return;
  }
  const int step = P.n / r;
  for (int p = 0; p < r; ++p) {
    for (int b = 0; b < B; ++b) y[p * ystride + b] = {0.0, 0.0};
    for (int q = 0; q < r; ++q) {
      const cd w = twiddle(P, (int)(((long long)p * q % r) * step), inv);
      for (int b = 0; b < B; ++b) {
        const cd v = cmul(t[q * B + b], w);
        y[p * ystride + b].re += v.re;
        y[p * ystride + b].im += v.im;
      }
    }
  }
}

// y[k] = sum_t x[t] w_n^{tk} for t, k in [0, n); x B-vectors at stride xs
// (in B-vectors), y contiguous; factors P.fac[fi..] multiply to n
void rec(const cd* x, size_t xs, cd* y, int n, int fi, const LinePlan& P, bool inv) {
  const int r = P.fac[fi];
  const int m = n / r;
  cd t[16 * B];
  std::vector<cd> big;
  cd* tt = t;
  if (r > 16) {
    big.resize((size_t)r * B);
    tt = big.data();
  }
  if (m == 1) {
    for (int q = 0; q < r; ++q)
      for (int b = 0; b < B; ++b) tt[q * B + b] = x[(size_t)q * xs * B + b];
    dft_small(tt, y, B, r, P, inv);
    return;
  }
  for (int q = 0; q < r; ++q) rec(x + (size_t)q * xs * B, xs * r, y + (size_t)q * m * B, m, fi + 1, P, inv);
  const int ws = P.n / n;
  for (int k = 0; k < m; ++k) {
    for (int b = 0; b < B; ++b) tt[b] = y[(size_t)k * B + b];
    for (int q = 1; q < r; ++q) {
      const cd w = twiddle(P, ws * q * k, inv);
      for (int b = 0; b < B; ++b) tt[q * B + b] = cmul(y[((size_t)q * m + k) * B + b], w);
    }
    dft_small(tt, y + (size_t)k * B, (size_t)m * B, r, P, inv);
  }
}

// transform B interleaved lines of length n held in `in` (n B-vectors) into `out`
void lines(const cd* in, cd* out, int n, bool inv) {
  if (n == 1) {
    std::memcpy(out, in, sizeof(cd) * B);
    return;
  }
  const LinePlan& P = line_plan(n);
  rec(in, 1, out, n, 0, P, inv);
}

enum Kind { R2C, C2R, C2C };

}  // namespace

struct fftw_plan_s {
  Kind kind;
  int n0, n1, n2;
  double* r;
  cd* c;
  cd* c2;
  int sign;
};

namespace {

// 2D part of a 3D transform on complex data [n0][n1][nc] (row stride nc):
// columns along n1 then n0 (forward) or n0 then n1 (inverse)
void columns(cd* data, int n0, int n1, int nc, bool inv) {
  auto along1 = [&]() {
#pragma omp parallel num_threads(nthreads())
    {
      std::vector<cd> a((size_t)n1 * B), o((size_t)n1 * B);
#pragma omp for schedule(static)
      for (long long task = 0; task < (long long)n0 * ((nc + B - 1) / B); ++task) {
        const int i = (int)(task / ((nc + B - 1) / B));
        const int c0 = (int)(task % ((nc + B - 1) / B)) * B;
        const int nb = std::min(B, nc - c0);
        for (int e = 0; e < n1; ++e) {
          const cd* src = data + ((size_t)i * n1 + e) * nc + c0;
          for (int b = 0; b < B; ++b) a[(size_t)e * B + b] = (b < nb) ? src[b] : cd{0.0, 0.0};
        }
        lines(a.data(), o.data(), n1, inv);
        for (int e = 0; e < n1; ++e) {
          cd* dst = data + ((size_t)i * n1 + e) * nc + c0;
          for (int b = 0; b < nb; ++b) dst[b] = o[(size_t)e * B + b];
        }
      }
    }
  };
  auto along0 = [&]() {
#pragma omp parallel num_threads(nthreads())
    {
      std::vector<cd> a((size_t)n0 * B), o((size_t)n0 * B);
#pragma omp for schedule(static)
      for (long long task = 0; task < (long long)n1 * ((nc + B - 1) / B); ++task) {
        const int j = (int)(task / ((nc + B - 1) / B));
        const int c0 = (int)(task % ((nc + B - 1) / B)) * B;
        const int nb = std::min(B, nc - c0);
        for (int e = 0; e < n0; ++e) {
          const cd* src = data + ((size_t)e * n1 + j) * nc + c0;
          for (int b = 0; b < B; ++b) a[(size_t)e * B + b] = (b < nb) ? src[b] : cd{0.0, 0.0};
        }
        lines(a.data(), o.data(), n0, inv);
        for (int e = 0; e < n0; ++e) {
          cd* dst = data + ((size_t)e * n1 + j) * nc + c0;
          for (int b = 0; b < nb; ++b) dst[b] = o[(size_t)e * B + b];
        }
      }
    }
  };
  if (!inv) {
    along1();
    along0();
  } else {
    along0();
    along1();
  }
}

// rows along n2 of a real array (row stride rs reals) into complex rows of
// n2/2+1 values (row stride nc complex); in place when r and c alias
void rows_r2c(const double* r, size_t rs, cd* c, size_t nc, long long nrows, int n2) {
  const int h = n2 / 2;
  const bool even = (n2 % 2 == 0);
  const LinePlan& P = line_plan(n2);
#pragma omp parallel num_threads(nthreads())
  {
    const int L = even ? h : n2;
    std::vector<cd> a((size_t)L * B), o((size_t)L * B);
#pragma omp for schedule(static)
    for (long long r0 = 0; r0 < nrows; r0 += B) {
      const int nb = (int)std::min<long long>(B, nrows - r0);
      for (int b = 0; b < B; ++b) {
        const double* x = r + (size_t)(r0 + b) * rs;
        for (int m = 0; m < L; ++m)
          a[(size_t)m * B + b] = (b >= nb) ? cd{0.0, 0.0} : (even ? cd{x[2 * m], x[2 * m + 1]} : cd{x[m], 0.0});
      }
      lines(a.data(), o.data(), L, false);
      for (int b = 0; b < nb; ++b) {
        cd* X = c + (size_t)(r0 + b) * nc;
        if (!even) {
          for (int k = 0; k <= h; ++k) X[k] = o[(size_t)k * B + b];
          continue;
        }
        for (int k = 0; k <= h; ++k) {
          const cd zk = o[(size_t)(k % h) * B + b];
          const cd zc = cconj(o[(size_t)((h - k) % h) * B + b]);
          const cd E = {0.5 * (zk.re + zc.re), 0.5 * (zk.im + zc.im)};
          // O = (zk - zc) / (2i)
          const cd O = {0.5 * (zk.im - zc.im), -0.5 * (zk.re - zc.re)};
          const cd wo = cmul(P.w[k % n2], O);
          X[k] = {E.re + wo.re, E.im + wo.im};
        }
      }
    }
  }
}

// inverse of rows_r2c: complex rows X[0..n2/2] (imaginary parts of the first
// and, for even n2, the last term ignored) into real rows
void rows_c2r(const cd* c, size_t nc, double* r, size_t rs, long long nrows, int n2) {
  const int h = n2 / 2;
  const bool even = (n2 % 2 == 0);
  const LinePlan& P = line_plan(n2);
#pragma omp parallel num_threads(nthreads())
  {
    const int L = even ? h : n2;
    std::vector<cd> a((size_t)L * B), o((size_t)L * B);
#pragma omp for schedule(static)
    for (long long r0 = 0; r0 < nrows; r0 += B) {
      const int nb = (int)std::min<long long>(B, nrows - r0);
      for (int b = 0; b < B; ++b) {
        if (b >= nb) {
          for (int m = 0; m < L; ++m) a[(size_t)m * B + b] = {0.0, 0.0};
          continue;
        }
        const cd* X = c + (size_t)(r0 + b) * nc;
        auto Xk = [&](int k) -> cd {
          cd v = X[k];
          if (k == 0 || (even && k == h)) v.im = 0.0;
          return v;
        };
        if (!even) {
          for (int k = 0; k < n2; ++k) a[(size_t)k * B + b] = (k <= h) ? Xk(k) : cconj(Xk(n2 - k));
          continue;
        }
        for (int k = 0; k < h; ++k) {
          const cd A = Xk(k), Bc = cconj(Xk(h - k));
          const cd E = {A.re + Bc.re, A.im + Bc.im};
          const cd D = {A.re - Bc.re, A.im - Bc.im};
          const cd O = cmul(D, cconj(P.w[k]));  // (A - B) e^{+2 pi i k / n2}
          a[(size_t)k * B + b] = {E.re - O.im, E.im + O.re};  // E + i O
        }
      }
      lines(a.data(), o.data(), L, true);
      for (int b = 0; b < nb; ++b) {
        double* x = r + (size_t)(r0 + b) * rs;
        if (!even) {
          for (int m = 0; m < n2; ++m) x[m] = o[(size_t)m * B + b].re;
          continue;
        }
        for (int m = 0; m < h; ++m) {
          x[2 * m] = o[(size_t)m * B + b].re;
          x[2 * m + 1] = o[(size_t)m * B + b].im;
        }
      }
    }
  }
}

// contiguous complex rows of length n2
void rows_c2c(const cd* in, cd* out, long long nrows, int n2, bool inv) {
#pragma omp parallel num_threads(nthreads())
  {
    std::vector<cd> a((size_t)n2 * B), o((size_t)n2 * B);
#pragma omp for schedule(static)
    for (long long r0 = 0; r0 < nrows; r0 += B) {
      const int nb = (int)std::min<long long>(B, nrows - r0);
      for (int b = 0; b < B; ++b)
        for (int m = 0; m < n2; ++m) a[(size_t)m * B + b] = (b < nb) ? in[(size_t)(r0 + b) * n2 + m] : cd{0.0, 0.0};
      lines(a.data(), o.data(), n2, inv);
      for (int b = 0; b < nb; ++b)
        for (int m = 0; m < n2; ++m) out[(size_t)(r0 + b) * n2 + m] = o[(size_t)m * B + b];
    }
  }
}

}  // namespace

extern "C" {

const char fftw_version[] = "project CPU transform behind an FFTW3 API shim (oracle/_ref)";

void* fftw_malloc(size_t n) {
  void* p = nullptr;
  if (posix_memalign(&p, 64, n ? n : 64) != 0) return nullptr;
  return p;
}

void fftw_free(void* p) { std::free(p); }

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned) {
  return new fftw_plan_s{R2C, n0, n1, n2, in, reinterpret_cast<cd*>(out), nullptr, -1};
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned) {
  return new fftw_plan_s{C2R, n0, n1, n2, out, reinterpret_cast<cd*>(in), nullptr, +1};
}

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
  return new fftw_plan_s{C2C, n0, n1, n2, nullptr, reinterpret_cast<cd*>(in), reinterpret_cast<cd*>(out), sign};
}

void fftw_execute(const fftw_plan p) {
  const int n0 = p->n0, n1 = p->n1, n2 = p->n2;
  const size_t nc = (size_t)n2 / 2 + 1;
  const long long nrows = (long long)n0 * n1;
  if (p->kind == R2C) {
    const bool inplace = reinterpret_cast<void*>(p->r) == reinterpret_cast<void*>(p->c);
    const size_t rs = inplace ? 2 * nc : (size_t)n2;
    rows_r2c(p->r, rs, p->c, nc, nrows, n2);
    columns(p->c, n0, n1, (int)nc, false);
  } else if (p->kind == C2R) {
    const bool inplace = reinterpret_cast<void*>(p->r) == reinterpret_cast<void*>(p->c);
    const size_t rs = inplace ? 2 * nc : (size_t)n2;
    columns(p->c, n0, n1, (int)nc, true);
    rows_c2r(p->c, nc, p->r, rs, nrows, n2);
  } else {
    const bool inv = p->sign > 0;
    rows_c2c(p->c, p->c2, nrows, n2, inv);
    columns(p->c2, n0, n1, n2, inv);
  }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) { g_threads = nthreads; }

void fftw_cleanup_threads(void) {}

}  // extern "C"
