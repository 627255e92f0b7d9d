// Fused prologue/epilogue functors for the FFT passes.
//
// Orszag 3/2 convolution (convolution.hh:513-668) without a padded grid in
// HBM: the padded spectrum is nonzero only in rows x (or y) in
// [0, N/2] U [N+1, M-1] and in kz <= N/2 (pad_insert, convolution.hh:575-590),
// so the c2r's x pass reads the N-grid field directly (Hessian factor, pad map
// and scale applied on load), the y pass reads the N compact rows, the z pass
// fuses both c2r's with the product and the r2c, and the r2c's x pass writes
// only the N rows that unpad keeps (convolution.hh:627-653), applying the
// Nyquist zeroing and the op:: output operator (operators.hh:25-35) on store.
#pragma once

#include "mf_fft.cuh"
#include "mf_plt_dev.cuh"

namespace mf {

enum OperandKind : int {
  OPND_PLAIN = 0,  // f
  OPND_HESS = 1,   // (i g_a)(i g_b) f
  OPND_SUM = 2,    // ((i g_a)(i g_b) + (i g_c)(i g_d)) f
  OPND_DIFF = 3,   // ((i g_a)(i g_b) - (i g_c)(i g_d)) f
  OPND_GRAD = 4,   // (i g_a) f
};

enum OutOp : int { OUT_ASSIGN = 0, OUT_ADD = 1, OUT_SUB = 2, OUT_AXPY = 3 };

// gradient factor g_d of Grid_FFT::gradient (grid_fft.hh:376-385): the
// component of k, zero on the Nyquist index.
template <typename T>
__device__ __forceinline__ T gradk(int idx, int n, T kfac) {
  return (idx != (n >> 1)) ? T(idx - ((idx > (n >> 1)) ? n : 0)) * kfac : T(0);
}
// get_k component (grid_fft.hh:281-296): Nyquist stays positive
template <typename T>
__device__ __forceinline__ T kcomp(int idx, int n, T kfac) {
  return T(idx - ((idx > (n >> 1)) ? n : 0)) * kfac;
}

template <typename T>
struct Operand {
  const cplx<T>* f;
  int kind;
  int d[4];
};

__device__ __forceinline__ int sel3(int d, int i, int j, int k) { return d == 0 ? i : (d == 1 ? j : k); }

// apply the operand's k-space factor to f at (i, j, kz)
template <typename T>
__device__ __forceinline__ cplx<T> operand_value(int kind, int d0, int d1, int d2, int d3, cplx<T> f, int i, int j,
                                                int kz, int n, T kfac) {
  if (kind == OPND_PLAIN) return f;
  if (kind == OPND_GRAD) {
    const T g = gradk<T>(sel3(d0, i, j, kz), n, kfac);
    return mkc<T>(-g * f.y, g * f.x);
  }
  const T h1 = -(gradk<T>(sel3(d0, i, j, kz), n, kfac) * gradk<T>(sel3(d1, i, j, kz), n, kfac));
  T h = h1;
  if (kind != OPND_HESS) {
    const T h2 = -(gradk<T>(sel3(d2, i, j, kz), n, kfac) * gradk<T>(sel3(d3, i, j, kz), n, kfac));
    h = (kind == OPND_SUM) ? (h1 + h2) : (h1 - h2);
  }
  return mkc<T>(h * f.x, h * f.y);
}

struct ConvGeom {
  int N;       // unpadded size
  int M;       // padded size (3N/2, or N for the aliased convolver)
  int Kz;      // N/2 + 1 stored kz columns
  bool orszag;
  // padded row index -> source row, -1 in the zero gap
  __device__ __forceinline__ int src_row(int x) const {
    if (!orszag) return x;
    if (x <= (N >> 1)) return x;
    if (x > N) return x - (N >> 1);
    return -1;
  }
  // padded row kept by unpad -> original row, -1 otherwise
  __device__ __forceinline__ int kept_row(int x) const { return src_row(x); }
};

// The same geometry as compile-time constants for a pass of length L over the
// padded axis (M = L): Orszag 3/2 (N = 2L/3) or the aliased convolver
// (N = L).  The strided passes are launched with it, so that their per-element
// row maps and addresses fold into immediates (about a quarter fewer
// instructions per element of the length-768 passes than with ConvGeom).
template <int L, bool ORSZAG>
struct CGeom {
  static constexpr int M = L;
  static constexpr int N = ORSZAG ? 2 * L / 3 : L;
  static constexpr int Kz = N / 2 + 1;
  static constexpr bool orszag = ORSZAG;
  __device__ __forceinline__ static constexpr int src_row(int x) {
    return !ORSZAG ? x : (x <= (N >> 1) ? x : (x > N ? x - (N >> 1) : -1));
  }
  __device__ __forceinline__ static constexpr int kept_row(int x) { return src_row(x); }
};
// a run-time geometry matching CGeom<L, ORSZAG>
template <class G>
inline bool geom_matches(const ConvGeom& g) {
  return g.orszag == G::orszag && g.M == G::M && g.N == G::N && g.Kz == G::Kz;
}

// x pass of the operands' c2r: slab = j, e = x in [0, M), col = kz.
// blockIdx.z selects the operand.
template <typename T, class G = ConvGeom>
struct ConvXInvOp {
  using C = cplx<T>;
  Operand<T> opnd[3];
  C* dst[3];  // work buffers [M][M][Kz]; rows j < N of each x slab
  G g;
  T kfac, scale;
  static constexpr bool kPrefetch = false;
  template <class G2>
  ConvXInvOp<T, G2> with_geom() const {
    ConvXInvOp<T, G2> o{};
    for (int k = 0; k < 3; ++k) {
      o.opnd[k] = opnd[k];
      o.dst[k] = dst[k];
    }
    o.kfac = kfac;
    o.scale = scale;
    return o;
  }
  // operand fields selected without dynamic indexing (keeps them in registers)
  template <int F>
  __device__ __forceinline__ int dsel(int z) const {
    return z == 0 ? opnd[0].d[F] : (z == 1 ? opnd[1].d[F] : opnd[2].d[F]);
  }
  __device__ __forceinline__ C load(int j, int x, int kz) const {
    const int i = g.src_row(x);
    if (i < 0) return mkc<T>(T(0), T(0));
    const int z = blockIdx.z;
    const C* f = z == 0 ? opnd[0].f : (z == 1 ? opnd[1].f : opnd[2].f);
    const int kind = z == 0 ? opnd[0].kind : (z == 1 ? opnd[1].kind : opnd[2].kind);
    const C v0 = f[((long long)i * g.N + j) * g.Kz + kz];
    const C v = operand_value<T>(kind, dsel<0>(z), dsel<1>(z), dsel<2>(z), dsel<3>(z), v0, i, j, kz, g.N, kfac);
    return mkc<T>(v.x * scale, v.y * scale);
  }
  __device__ __forceinline__ void store(int j, int x, int kz, C v) const {
    const int z = blockIdx.z;
    C* d = z == 0 ? dst[0] : (z == 1 ? dst[1] : dst[2]);
    d[((long long)x * g.M + j) * g.Kz + kz] = v;
  }
  // pipelined form (k_colfft_pipe): raw source element and on-read transform; z = operand
  static constexpr bool kPipe = true;
  __device__ __forceinline__ const C* srcp(int z, int j, int x, int kz) const {
    const int i = g.src_row(x);
    if (i < 0) return nullptr;
    const C* f = z == 0 ? opnd[0].f : (z == 1 ? opnd[1].f : opnd[2].f);
    return f + ((long long)i * g.N + j) * g.Kz + kz;
  }
  __device__ __forceinline__ C xform(int z, int j, int x, int kz, C v0) const {
    const int i = g.src_row(x);
    const int kind = z == 0 ? opnd[0].kind : (z == 1 ? opnd[1].kind : opnd[2].kind);
    const C v = operand_value<T>(kind, dsel<0>(z), dsel<1>(z), dsel<2>(z), dsel<3>(z), v0, i, j, kz, g.N, kfac);
    return mkc<T>(v.x * scale, v.y * scale);
  }
  // per-tile form: along x only g_i varies, so the operand factor (times the
  // scale) is the polynomial c0 + c1 g_i + c2 g_i^2 with coefficients fixed
  // by the operand kind, its directions, g_j and g_kz; GRAD multiplies by
  // i (c0 + c1 g_i)
  struct Tile {
    T c0, c1, c2;
    bool grad;
  };
  __device__ __forceinline__ Tile tile_prep(int z, int j, int kz) const {
    const int kind = z == 0 ? opnd[0].kind : (z == 1 ? opnd[1].kind : opnd[2].kind);
    const int d[4] = {dsel<0>(z), dsel<1>(z), dsel<2>(z), dsel<3>(z)};
    const T gj = gradk<T>(j, g.N, kfac), gk = gradk<T>(kz, g.N, kfac);
    auto gof = [&](int a) { return a == 1 ? gj : gk; };
    Tile t{T(0), T(0), T(0), false};
    auto term = [&](int a, int b, T sgn) {  // adds sgn * (-g_a g_b)
      const int m = (a == 0) + (b == 0);
      if (m == 2) t.c2 -= sgn;
      else if (m == 1) t.c1 -= sgn * gof(a == 0 ? b : a);
      else t.c0 -= sgn * gof(a) * gof(b);
    };
    if (kind == OPND_PLAIN) {
      t.c0 = T(1);
    } else if (kind == OPND_GRAD) {
      t.grad = true;
      if (d[0] == 0) t.c1 = T(1);
      else t.c0 = gof(d[0]);
    } else {
      term(d[0], d[1], T(1));
      if (kind == OPND_SUM) term(d[2], d[3], T(1));
      if (kind == OPND_DIFF) term(d[2], d[3], T(-1));
    }
    t.c0 *= scale;
    t.c1 *= scale;
    t.c2 *= scale;
    return t;
  }
  __device__ __forceinline__ C xform_tile(const Tile& t, int x, C v0) const {
    const T gi = gradk<T>(g.src_row(x), g.N, kfac);
    if (t.grad) {
      const T f = t.c1 * gi + t.c0;
      return mkc<T>(-f * v0.y, f * v0.x);
    }
    const T f = (t.c2 * gi + t.c1) * gi + t.c0;
    return mkc<T>(v0.x * f, v0.y * f);
  }
  __device__ __forceinline__ void store_z(int z, int j, int x, int kz, C v) const {
    C* d = z == 0 ? dst[0] : (z == 1 ? dst[1] : dst[2]);
    d[((long long)x * g.M + j) * g.Kz + kz] = v;
  }
};

// y pass of the operands' c2r: slab = x in [0,M), e = y in [0,M), col = kz
template <typename T, class G = ConvGeom>
struct ConvYInvOp {
  using C = cplx<T>;
  const C* src[3];  // work buffers, compact rows j < N of each x slab
  C* dst[3];        // same buffers, rows y < M (in place per slab)
  G g;
  static constexpr bool kPrefetch = false;
  template <class G2>
  ConvYInvOp<T, G2> with_geom() const {
    ConvYInvOp<T, G2> o{};
    for (int k = 0; k < 3; ++k) {
      o.src[k] = src[k];
      o.dst[k] = dst[k];
    }
    return o;
  }
  static constexpr bool kColSwizzle = true;  // bank-conflict-free exchange rows (registers to spare)
  __device__ __forceinline__ C load(int x, int y, int kz) const {
    const int j = g.src_row(y);
    if (j < 0) return mkc<T>(T(0), T(0));
    const int z = blockIdx.z;
    const C* s = z == 0 ? src[0] : (z == 1 ? src[1] : src[2]);
    return s[((long long)x * g.M + j) * g.Kz + kz];
  }
  __device__ __forceinline__ void store(int x, int y, int kz, C v) const {
    const int z = blockIdx.z;
    C* d = z == 0 ? dst[0] : (z == 1 ? dst[1] : dst[2]);
    d[((long long)x * g.M + y) * g.Kz + kz] = v;
  }
  static constexpr bool kPipe = true;
  __device__ __forceinline__ const C* srcp(int z, int x, int y, int kz) const {
    const int j = g.src_row(y);
    if (j < 0) return nullptr;
    const C* s0 = z == 0 ? src[0] : (z == 1 ? src[1] : src[2]);
    return s0 + ((long long)x * g.M + j) * g.Kz + kz;
  }
  __device__ __forceinline__ C xform(int, int, int, int, C v) const { return v; }
  __device__ __forceinline__ void store_z(int z, int x, int y, int kz, C v) const {
    C* d = z == 0 ? dst[0] : (z == 1 ? dst[1] : dst[2]);
    d[((long long)x * g.M + y) * g.Kz + kz] = v;
  }
};

// y pass of the product's r2c: keeps only the rows unpad reads
template <typename T, class G = ConvGeom>
struct ConvYFwdOp {
  using C = cplx<T>;
  const C* src;  // work buffer, rows y < M
  C* dst;        // same buffer, compact rows j < N (in place per slab)
  G g;
  static constexpr bool kPrefetch = false;
  template <class G2>
  ConvYFwdOp<T, G2> with_geom() const {
    ConvYFwdOp<T, G2> o{};
    o.src = src;
    o.dst = dst;
    return o;
  }
  static constexpr bool kColSwizzle = true;  // bank-conflict-free exchange rows (registers to spare)
  __device__ __forceinline__ C load(int x, int y, int kz) const {
    return src[((long long)x * g.M + y) * g.Kz + kz];
  }
  __device__ __forceinline__ void store(int x, int y, int kz, C v) const {
    const int j = g.kept_row(y);
    if (j >= 0) dst[((long long)x * g.M + j) * g.Kz + kz] = v;
  }
  static constexpr bool kPipe = true;
  __device__ __forceinline__ const C* srcp(int, int x, int y, int kz) const {
    return src + ((long long)x * g.M + y) * g.Kz + kz;
  }
  __device__ __forceinline__ C xform(int, int, int, int, C v) const { return v; }
  __device__ __forceinline__ void store_z(int, int x, int y, int kz, C v) const { store(x, y, kz, v); }
};

// x pass of the product's r2c + unpad + output operator (+ optional inverse
// Laplacian of the accumulated target, grid_fft.hh:440-449)
template <typename T, class G = ConvGeom>
struct ConvXFwdOp {
  using C = cplx<T>;
  const C* src;  // work buffer, compact rows j < N
  C* target;     // N-grid k-space [N][N][Kz]
  G g;
  T scale;       // FFT norm / unpad factor
  int out_op;
  T x;           // multiply_add_to factor
  int post_invlap;
  T kfac;
  template <class G2>
  ConvXFwdOp<T, G2> with_geom() const {
    ConvXFwdOp<T, G2> o{};
    o.src = src;
    o.target = target;
    o.scale = scale;
    o.out_op = out_op;
    o.x = x;
    o.post_invlap = post_invlap;
    o.kfac = kfac;
    return o;
  }
  // the read-modify-write target is fetched before the transform so its
  // latency overlaps the FFT
  static constexpr bool kPrefetch = true;
  __device__ __forceinline__ C load(int j, int xx, int kz) const {
    return src[((long long)xx * g.M + j) * g.Kz + kz];
  }
  __device__ __forceinline__ C prefetch(int j, int xx, int kz) const {
    const int i = g.kept_row(xx);
    if (i < 0 || out_op == OUT_ASSIGN) return mkc<T>(T(0), T(0));
    return target[((long long)i * g.N + j) * g.Kz + kz];
  }
  __device__ __forceinline__ void store_pre(int j, int xx, int kz, C v, C r) const {
    const int i = g.kept_row(xx);
    if (i < 0) return;
    const int nh = g.N >> 1;
    v = mkc<T>(v.x * scale, v.y * scale);
    if (g.orszag && (i == nh || j == nh || kz == nh)) v = mkc<T>(T(0), T(0));
    const long long idx = ((long long)i * g.N + j) * g.Kz + kz;
    if (out_op == OUT_ASSIGN) r = v;
    else if (out_op == OUT_ADD) r = cadd(r, v);
    else if (out_op == OUT_SUB) r = csub(r, v);
    else r = mkc<T>(r.x + v.x * x, r.y + v.y * x);
    if (post_invlap) {
      const T kx = kcomp<T>(i, g.N, kfac), ky = kcomp<T>(j, g.N, kfac), kzz = kcomp<T>(kz, g.N, kfac);
      const T k2 = kx * kx + ky * ky + kzz * kzz;
      const T m = -rcp_rn(k2);
      r = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(r.x * m, r.y * m);
    }
    target[idx] = r;
  }
  __device__ __forceinline__ void store(int j, int xx, int kz, C v) const { store_pre(j, xx, kz, v, prefetch(j, xx, kz)); }
  static constexpr bool kPipe = true;
  __device__ __forceinline__ const C* srcp(int, int j, int xx, int kz) const {
    return src + ((long long)xx * g.M + j) * g.Kz + kz;
  }
  __device__ __forceinline__ C xform(int, int, int, int, C v) const { return v; }
  __device__ __forceinline__ void store_z(int, int j, int xx, int kz, C v) const { store(j, xx, kz, v); }
};

// Sub-lattice phase chain: the shift_field calls (grid_fft.hh:832-842) that
// set_positions / set_velocities / set_masses (particle_generator.hh:369-639)
// apply in sequence, each a shift dS of the field by a fraction of a cell.
// Shifts are in quarter cells (s4 = 4 dS: the relative sub-lattice shifts are
// multiples of 1/2, the secondary-lattice shift of RSC is 1/4), the phases
// exp(i dS.k dx) are read from an exact table exp(+2 pi i m / 4n).
template <typename T>
struct ShiftChain {
  using C = cplx<T>;
  const C* phase;  // 4n entries exp(+2 pi i m / 4n)
  int nstep;
  int s4[8][3];
  // phase of step s at (i, j, kz), k = get_k (Nyquist index positive)
  __device__ __forceinline__ C step_phase(int s, int n, int i, int j, int kz) const {
    const int ii = i - ((i > (n >> 1)) ? n : 0), jj = j - ((j > (n >> 1)) ? n : 0);
    int m = (s4[s][0] * ii + s4[s][1] * jj + s4[s][2] * kz) % (4 * n);
    if (m < 0) m += 4 * n;
    return phase[m];
  }
  // Apply the chain to K values v at (i, j, kz).  The reference re-projects
  // onto real fields (r2c of the c2r) before every shift; on the kz = 0 and
  // kz = n/2 planes that projection pairs k with -k, H(X)(k) = (X(k) +
  // conj X(-k)) / 2, so there vm must hold the values at (-i, -j, kz).
  template <int K>
  __device__ __forceinline__ void apply(int n, int i, int j, int kz, C (&v)[K], C (&vm)[K]) const {
    if (kz == 0 || kz == (n >> 1)) {
      const int im = (n - i) % n, jm = (n - j) % n;
      for (int s = 0; s < nstep; ++s) {
        const C pk = step_phase(s, n, i, j, kz), pm = step_phase(s, n, im, jm, kz);
#pragma unroll
        for (int d = 0; d < K; ++d) {
          const C hk = mkc<T>(T(0.5) * (v[d].x + vm[d].x), T(0.5) * (v[d].y - vm[d].y));
          const C hm = mkc<T>(T(0.5) * (vm[d].x + v[d].x), T(0.5) * (vm[d].y - v[d].y));
          v[d] = cmul(hk, pk);
          vm[d] = cmul(hm, pm);
        }
      }
      return;
    }
    for (int s = 0; s < nstep; ++s) {
      const C ph = step_phase(s, n, i, j, kz);
#pragma unroll
      for (int d = 0; d < K; ++d) v[d] = cmul(v[d], ph);
    }
  }
};

// x pass of the c2r of one displacement / velocity component, with the
// k-space assembly of ic_generator.cc:829-858 / :884-931 fused into the load:
//   i g_d phitot + w_A (i g_d' A3[d''] - i g_d'' A3[d']), times unit/L, zero DC,
// times the sub-lattice phase chain (ShiftChain).
// slab = j, e = i, col = kz; in place on the destination grid.
template <typename T>
struct AssembleXInvOp {
  using C = cplx<T>;
  const C* phitot;  // growth-weighted order sum (FP64 sum stored in T)
  const C* A3p;     // A3[d'] (nullptr below 3LPT)
  const C* A3pp;    // A3[d'']
  C* dst;
  int n, Kz, d;
  ShiftChain<T> ch;
  T kfac, unit;
  const double* wA;  // device scalar: weight of the A3 term (growth factor of this pass)
  int plt;          // PLT corrected gradient (lattice_gradient, particle_plt.hh:551-573)
  int vel;          // velocities: times the PLT growth-rate correction vfac_corr (:575-585)
  PLTDev<T> P;
  const T* pg;  // tabulated PLT gradient and vfac_corr [idx][4] (nullptr: evaluate from P)
  static constexpr bool kPrefetch = false;
  static constexpr bool kPipe = false;

  // k-space combination at (i, j, kz) before any sub-lattice phase
  __device__ __forceinline__ C assemble(int i, int j, int kz) const {
    const long long idx = ((long long)i * n + j) * Kz + kz;
    if (idx == 0) return mkc<T>(T(0), T(0));
    const int dp = (d + 1) % 3, dpp = (d + 2) % 3;
    T gd, gp, gpp, vc = T(1);
    if (plt) {
      T g[3];
      if (pg) {
        const T* q = pg + 4 * idx;
        g[0] = q[0];
        g[1] = q[1];
        g[2] = q[2];
        if (vel) vc = q[3];
      } else {
        plt_gradient<T>(P, i, j, kz, g, vel ? &vc : nullptr);
      }
      gd = (d == 0) ? g[0] : ((d == 1) ? g[1] : g[2]);
      gp = (dp == 0) ? g[0] : ((dp == 1) ? g[1] : g[2]);
      gpp = (dpp == 0) ? g[0] : ((dpp == 1) ? g[1] : g[2]);
    } else {
      gd = gradk<T>(sel3(d, i, j, kz), n, kfac);
      gp = gradk<T>(sel3(dp, i, j, kz), n, kfac);
      gpp = gradk<T>(sel3(dpp, i, j, kz), n, kfac);
    }
    const C P1 = phitot[idx];
    T rr = -gd * P1.y, ri = gd * P1.x;
    if (A3p) {
      const C X1 = A3pp[idx], X2 = A3p[idx];
      const T w = T(__ldg(wA));
      rr += w * (-(gp * X1.y) + gpp * X2.y);
      ri += w * (gp * X1.x - gpp * X2.x);
    }
    if (plt && vel) {
      rr *= vc;
      ri *= vc;
    }
    return mkc<T>(rr * unit, ri * unit);
  }
  __device__ __forceinline__ C load(int j, int i, int kz) const {
    C v[1] = {assemble(i, j, kz)};
    if (ch.nstep == 0) return v[0];
    C vm[1] = {mkc<T>(T(0), T(0))};
    if (kz == 0 || kz == (n >> 1)) vm[0] = assemble((n - i) % n, (n - j) % n, kz);
    ch.template apply<1>(n, i, j, kz, v, vm);
    return v[0];
  }
  __device__ __forceinline__ void store(int j, int i, int kz, C v) const { dst[((long long)i * n + j) * Kz + kz] = v; }
};

// convolve3's intermediate truncation on a work buffer, in place: the x pass
// of the pair product's r2c, the unpad to the N-cube with the Nyquist planes
// zeroed (convolution.hh:618-653, op::assign_to), and the x pass of the
// truncated field's padded c2r (pad_insert, convolution.hh:570-592) — the
// unpadded N-grid never leaves the tile.  slab = j < N, e = x in [0, M), col = kz
template <typename T, class G = ConvGeom>
struct ConvXTruncOp {
  using C = cplx<T>;
  C* buf;  // work buffer, compact rows j < N of each x slab
  G g;
  T scale_out, scale_in;  // the unpad factor of the r2c, the pad factor of the c2r
  template <class G2>
  ConvXTruncOp<T, G2> with_geom() const {
    ConvXTruncOp<T, G2> o{};
    o.buf = buf;
    o.scale_out = scale_out;
    o.scale_in = scale_in;
    return o;
  }
  __device__ __forceinline__ C* at(int j, int x, int kz) const { return buf + ((long long)x * g.M + j) * g.Kz + kz; }
  __device__ __forceinline__ C mask(int j, int x, int kz, C v) const {
    const int i = g.kept_row(x);
    const int nh = g.N >> 1;
    if (i < 0 || (g.orszag && (i == nh || j == nh || kz == nh))) return mkc<T>(T(0), T(0));
    v = mkc<T>(v.x * scale_out, v.y * scale_out);  // the unpadded value
    return mkc<T>(v.x * scale_in, v.y * scale_in);  // the padded operand
  }
};

// plain strided pass over an n-grid: element (slab, e, col) at
// base[slab*slab_str + e*e_str + col]; in place, scale on store.  AXIS 0 / 1
// with the pass length L: the strides of an x / y pass over an L-grid as
// compile-time constants (e_str, slab_str = L Kz, Kz or Kz, L Kz with
// Kz = L/2 + 1); AXIS -1: the run-time strides
template <typename T, int L = 0, int AXIS = -1>
struct PlainStridedOp {
  using C = cplx<T>;
  C* p;
  long long e_str, slab_str;
  T scale;
  static constexpr bool kPrefetch = false;
  static constexpr long long KZ = L / 2 + 1;
  __device__ __forceinline__ long long es() const {
    if constexpr (AXIS == 0) return (long long)L * KZ;
    else if constexpr (AXIS == 1) return KZ;
    else return e_str;
  }
  __device__ __forceinline__ long long ss() const {
    if constexpr (AXIS == 0) return KZ;
    else if constexpr (AXIS == 1) return (long long)L * KZ;
    else return slab_str;
  }
  // the op with compile-time strides when they are those of an x (0) or y (1)
  // pass over an L2-grid
  template <int L2, int AX2>
  PlainStridedOp<T, L2, AX2> with_axis() const {
    return PlainStridedOp<T, L2, AX2>{p, e_str, slab_str, scale};
  }
  __device__ __forceinline__ C load(int slab, int e, int col) const {
    return p[(long long)slab * ss() + (long long)e * es() + col];
  }
  __device__ __forceinline__ void store(int slab, int e, int col, C v) const {
    p[(long long)slab * ss() + (long long)e * es() + col] = mkc<T>(v.x * scale, v.y * scale);
  }
  static constexpr bool kPipe = true;
  __device__ __forceinline__ const C* srcp(int, int slab, int e, int col) const {
    return p + (long long)slab * ss() + (long long)e * es() + col;
  }
  __device__ __forceinline__ C xform(int, int, int, int, C v) const { return v; }
  __device__ __forceinline__ void store_z(int, int slab, int e, int col, C v) const { store(slab, e, col, v); }
};

// plain z pass on the in-place padded layout: line = i*n + j, row of n+2 reals
template <typename T>
struct PlainZOp {
  using C = cplx<T>;
  T* p;
  int n;
  T scale;
  __device__ __forceinline__ C load_pair(int line, int m) const {
    return reinterpret_cast<const C*>(p + (long long)line * (n + 2))[m];
  }
  __device__ __forceinline__ void store(int line, int k, C v) const {
    reinterpret_cast<C*>(p + (long long)line * (n + 2))[k] = mkc<T>(v.x * scale, v.y * scale);
  }
  __device__ __forceinline__ C load(int line, int k) const {
    return reinterpret_cast<const C*>(p + (long long)line * (n + 2))[k];
  }
  __device__ __forceinline__ void store_pair(int line, int m, C v) const {
    reinterpret_cast<C*>(p + (long long)line * (n + 2))[m] = mkc<T>(v.x * scale, v.y * scale);
  }
};

// Shared-source form of the Orszag convolutions: every padded operand field
// is transformed to real space once and kept in HBM as lines of M reals,
// stored as H = M/2 packed pairs [line][H], line = x*M + y.

// the x pass of all three displacement / velocity components of one
// sub-lattice in one launch: the same k-space combination and sub-lattice
// phase chain as AssembleXInvOp, with the order sum, the three A3 fields and
// the gradient read once per mode for the three components
template <typename T, int NN = 0>
struct Assemble3XInvOp {
  using C = cplx<T>;
  const C* phitot;
  const C* A3[3];  // nullptr below 3LPT
  C* dst[3];
  int n, Kz;
  ShiftChain<T> ch;
  T kfac, unit;
  const double* wA;
  int plt, vel;
  const T* pg;  // tabulated PLT gradient and vfac_corr [idx][4]
  // grid size: NN when the op is specialised to a compile-time n (with_n)
  __device__ __forceinline__ int nn() const { return NN ? NN : n; }
  __device__ __forceinline__ int kzn() const { return NN ? NN / 2 + 1 : Kz; }
  template <int N2>
  Assemble3XInvOp<T, N2> with_n() const {
    Assemble3XInvOp<T, N2> o{};
    o.phitot = phitot;
    for (int d = 0; d < 3; ++d) {
      o.A3[d] = A3[d];
      o.dst[d] = dst[d];
    }
    o.n = n;
    o.Kz = Kz;
    o.ch = ch;
    o.kfac = kfac;
    o.unit = unit;
    o.wA = wA;
    o.plt = plt;
    o.vel = vel;
    o.pg = pg;
    return o;
  }
  __device__ __forceinline__ void assemble(int i, int j, int kz, C (&o)[3]) const {
    const int n = nn(), Kz = kzn();
    const long long idx = ((long long)i * n + j) * Kz + kz;
    if (idx == 0) {
      o[0] = o[1] = o[2] = mkc<T>(T(0), T(0));
      return;
    }
    T g[3], vc = T(1);
    if (plt) {
      const T* q = pg + 4 * idx;
      g[0] = q[0];
      g[1] = q[1];
      g[2] = q[2];
      if (vel) vc = q[3];
    } else {
      g[0] = gradk<T>(i, n, kfac);
      g[1] = gradk<T>(j, n, kfac);
      g[2] = gradk<T>(kz, n, kfac);
    }
    const C P1 = phitot[idx];
    C X[3] = {mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0))};
    T w = T(0);
    if (A3[0]) {
      X[0] = A3[0][idx];
      X[1] = A3[1][idx];
      X[2] = A3[2][idx];
      w = T(__ldg(wA));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int dp = (d + 1) % 3, dpp = (d + 2) % 3;
      T rr = -g[d] * P1.y, ri = g[d] * P1.x;
      if (A3[0]) {
        rr += w * (-(g[dp] * X[dpp].y) + g[dpp] * X[dp].y);
        ri += w * (g[dp] * X[dpp].x - g[dpp] * X[dp].x);
      }
      if (plt && vel) {
        rr *= vc;
        ri *= vc;
      }
      o[d] = mkc<T>(rr * unit, ri * unit);
    }
  }
  // slab = j, e = i, col = kz
  __device__ __forceinline__ void load3(int j, int i, int kz, C (&v)[3]) const {
    const int n = nn();
    assemble(i, j, kz, v);
    if (ch.nstep == 0) return;
    C vm[3];
    if (kz == 0 || kz == (n >> 1)) assemble((n - i) % n, (n - j) % n, kz, vm);
    ch.template apply<3>(n, i, j, kz, v, vm);
  }
  __device__ __forceinline__ void store(int d, int j, int i, int kz, C v) const {
    dst[d][((long long)i * nn() + j) * kzn() + kz] = v;
  }
};

// arguments of the fused z c2r + lattice readout (mf_kernels.cuh, k_zc2r3_lattice)
struct Lattice3Args {
  const void* comp[3];
  void* dst;
  const double* q;  // q[d*n + idx_d], lattice coordinates times the unit
  const float2* qf; // the same as float pairs (hi, lo) for FP32 positions
  int n, nlines, ishift, with_q, fields_mode;
  double norm;      // 1/sqrt(n^3) of the c2r
};

// z pass c2r of a work-buffer line [line][Kz] (kz > N/2 zero) into a real line
template <typename T>
struct PadC2RZOp {
  using C = cplx<T>;
  const C* src;
  long long src_stride;  // Kz
  C* dst;
  int H;
  __device__ __forceinline__ C load(int line, int k) const { return src[(long long)line * src_stride + k]; }
  __device__ __forceinline__ void store_pair(int line, int m, C v) const { dst[(long long)line * H + m] = v; }
};

// z pass r2c of one real padded field, keeping kz < kout
template <typename T>
struct PadR2CZOp {
  using C = cplx<T>;
  const C* src;
  int H;
  C* dst;
  long long dst_stride;  // Kz
  __device__ __forceinline__ C load_pair(int line, int m) const { return src[(long long)line * H + m]; }
  __device__ __forceinline__ void store(int line, int k, C v) const { dst[line * dst_stride + k] = v; }
};

// arguments of the fused Orszag z pass (mf_kernels.cuh, k_zconv)
template <typename T>
struct ZConvArgs {
  const cplx<T>* in[3];   // operand line arrays [line][kin]
  cplx<T>* out;           // product spectrum [line][kout]
  int nop;
  int kin;                // nonzero kz count of the operands (N/2+1)
  int kout;               // stored kz count (N/2+1)
  long long in_stride;    // complex elements between consecutive lines
  long long out_stride;
  int nlines;
  T out_scale;
  int* err;               // device error flag (bounded waits), may be null
};

}  // namespace mf
