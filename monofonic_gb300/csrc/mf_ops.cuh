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

// apply the operand's k-space factor to f at (i, j, kz)
template <typename T>
__device__ __forceinline__ cplx<T> operand_value(const Operand<T>& o, cplx<T> f, int i, int j, int kz, int n, T kfac) {
  if (o.kind == OPND_PLAIN) return f;
  const int ijk[3] = {i, j, kz};
  if (o.kind == OPND_GRAD) {
    const T g = gradk<T>(ijk[o.d[0]], n, kfac);
    return mkc<T>(-g * f.y, g * f.x);
  }
  const T h1 = -(gradk<T>(ijk[o.d[0]], n, kfac) * gradk<T>(ijk[o.d[1]], n, kfac));
  T h = h1;
  if (o.kind != OPND_HESS) {
    const T h2 = -(gradk<T>(ijk[o.d[2]], n, kfac) * gradk<T>(ijk[o.d[3]], n, kfac));
    h = (o.kind == OPND_SUM) ? (h1 + h2) : (h1 - h2);
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

// x pass of the operands' c2r: slab = j, e = x in [0, M), col = kz.
// blockIdx.z selects the operand.
template <typename T>
struct ConvXInvOp {
  using C = cplx<T>;
  Operand<T> opnd[3];
  C* dst[3];  // work buffers [M][M][Kz]; rows j < N of each x slab
  ConvGeom g;
  T kfac, scale;
  __device__ __forceinline__ C load(int j, int x, int kz) const {
    const int i = g.src_row(x);
    if (i < 0) return mkc<T>(T(0), T(0));
    const Operand<T>& o = opnd[blockIdx.z];
    const C f = o.f[((long long)i * g.N + j) * g.Kz + kz];
    const C v = operand_value<T>(o, f, i, j, kz, g.N, kfac);
    return mkc<T>(v.x * scale, v.y * scale);
  }
  __device__ __forceinline__ void store(int j, int x, int kz, C v) const {
    dst[blockIdx.z][((long long)x * g.M + j) * g.Kz + kz] = v;
  }
};

// y pass of the operands' c2r: slab = x in [0,M), e = y in [0,M), col = kz
template <typename T>
struct ConvYInvOp {
  using C = cplx<T>;
  const C* src[3];  // work buffers, compact rows j < N of each x slab
  C* dst[3];        // same buffers, rows y < M (in place per slab)
  ConvGeom g;
  __device__ __forceinline__ C load(int x, int y, int kz) const {
    const int j = g.src_row(y);
    if (j < 0) return mkc<T>(T(0), T(0));
    return src[blockIdx.z][((long long)x * g.M + j) * g.Kz + kz];
  }
  __device__ __forceinline__ void store(int x, int y, int kz, C v) const {
    dst[blockIdx.z][((long long)x * g.M + y) * g.Kz + kz] = v;
  }
};

// y pass of the product's r2c: keeps only the rows unpad reads
template <typename T>
struct ConvYFwdOp {
  using C = cplx<T>;
  const C* src;  // work buffer, rows y < M
  C* dst;        // same buffer, compact rows j < N (in place per slab)
  ConvGeom g;
  __device__ __forceinline__ C load(int x, int y, int kz) const {
    return src[((long long)x * g.M + y) * g.Kz + kz];
  }
  __device__ __forceinline__ void store(int x, int y, int kz, C v) const {
    const int j = g.kept_row(y);
    if (j >= 0) dst[((long long)x * g.M + j) * g.Kz + kz] = v;
  }
};

// x pass of the product's r2c + unpad + output operator (+ optional inverse
// Laplacian of the accumulated target, grid_fft.hh:440-449)
template <typename T>
struct ConvXFwdOp {
  using C = cplx<T>;
  const C* src;  // work buffer, compact rows j < N
  C* target;     // N-grid k-space [N][N][Kz]
  ConvGeom g;
  T scale;       // FFT norm / unpad factor
  int out_op;
  T x;           // multiply_add_to factor
  int post_invlap;
  T kfac;
  __device__ __forceinline__ C load(int j, int xx, int kz) const {
    return src[((long long)xx * g.M + j) * g.Kz + kz];
  }
  __device__ __forceinline__ void store(int j, int xx, int kz, C v) const {
    const int i = g.kept_row(xx);
    if (i < 0) return;
    const int nh = g.N >> 1;
    v = mkc<T>(v.x * scale, v.y * scale);
    if (g.orszag && (i == nh || j == nh || kz == nh)) v = mkc<T>(T(0), T(0));
    const long long idx = ((long long)i * g.N + j) * g.Kz + kz;
    C r;
    if (out_op == OUT_ASSIGN) r = v;
    else {
      r = target[idx];
      if (out_op == OUT_ADD) r = cadd(r, v);
      else if (out_op == OUT_SUB) r = csub(r, v);
      else r = mkc<T>(r.x + v.x * x, r.y + v.y * x);
    }
    if (post_invlap) {
      const T kx = kcomp<T>(i, g.N, kfac), ky = kcomp<T>(j, g.N, kfac), kzz = kcomp<T>(kz, g.N, kfac);
      const T k2 = kx * kx + ky * ky + kzz * kzz;
      r = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(-r.x / k2, -r.y / k2);
    }
    target[idx] = r;
  }
};

// plain strided pass over an n-grid: element (slab, e, col) at
// base[slab*slab_str + e*e_str + col]; in place, scale on store
template <typename T>
struct PlainStridedOp {
  using C = cplx<T>;
  C* p;
  long long e_str, slab_str;
  T scale;
  __device__ __forceinline__ C load(int slab, int e, int col) const {
    return p[(long long)slab * slab_str + (long long)e * e_str + col];
  }
  __device__ __forceinline__ void store(int slab, int e, int col, C v) const {
    p[(long long)slab * slab_str + (long long)e * e_str + col] = mkc<T>(v.x * scale, v.y * scale);
  }
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
};

}  // namespace mf
