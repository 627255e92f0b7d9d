// Device FFT machinery for the nLPT field pipeline (sm_103a).
//
// A line FFT of compile-time length L = 2^a 3^b is a Stockham auto-sort
// decimation-in-time transform.  Every thread of a line owns E = L/TPL
// elements in registers; each stage is a set of radix-R butterflies computed
// in registers, and consecutive stages exchange data through shared memory.
// The first stage reads its inputs through a caller-supplied loader and the
// last stage hands its outputs to a caller-supplied storer, so padding,
// Hessian factors, products, unpadding and output operators fuse into the
// FFT's global-memory loads and stores.
//
// Stage s (radix R, Lc = product of earlier radices), butterfly b in [0,L/R):
//   k = b mod Lc; x_p = in[b + p L/R] * w_L^(p k L/(Lc R)); X = DFT_R(x);
//   out[(b-k) R + k + q Lc] = X_q.
// Stage-0 inputs are in[b + p L/R0]; last-stage outputs are out[b + q L/Rl].
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace mf {

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename T> using cplx = typename cplx_of<T>::type;

template <typename T>
__host__ __device__ __forceinline__ cplx<T> mkc(T x, T y) { cplx<T> r; r.x = x; r.y = y; return r; }
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// complex products with one fused multiply-add per component (the build
// compiles with FP contraction off, which the float-pair arithmetic below
// needs; here the fusion is explicit)
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
#ifndef MF_FFT_FMA
#define MF_FFT_FMA 1
#endif
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  if (MF_FFT_FMA) {
    r.x = fma_rn(a.x, b.x, -(a.y * b.y));
    r.y = fma_rn(a.x, b.y, a.y * b.x);
  } else {
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
  }
  return r;
}
// a * conj(b)
template <typename C>
__device__ __forceinline__ C cmulc(C a, C b) {
  C r;
  if (MF_FFT_FMA) {
    r.x = fma_rn(a.x, b.x, a.y * b.y);
    r.y = fma_rn(a.y, b.x, -(a.x * b.y));
  } else {
    r.x = a.x * b.x + a.y * b.y;
    r.y = a.y * b.x - a.x * b.y;
  }
  return r;
}
template <typename C, typename T>
__device__ __forceinline__ C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C>
__device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
// correctly rounded reciprocal (IEEE round-to-nearest)
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }
// multiply by -i (forward) or +i (inverse)
// Float-pair ("double-float") arithmetic on the FP32 pipes, where GB300's
// FP64 rate would bound a streaming kernel.  A double value v is carried as
// the unevaluated pair (hi, lo) = (RN(v), RN(v - RN(v))), ~48 significant bits.
// q + psi rounded to float for a pair q and a float psi: TwoSum of q.hi and
// psi (exact), then the low parts; the result is the float nearest to the
// exact sum except when that sum lies within ~2^-24 ulp of a tie.
__device__ __forceinline__ float ff_add_q(float2 q, float psi) {
  const float s = q.x + psi;
  const float bb = s - q.x;
  const float e = (q.x - (s - bb)) + (psi - bb);
  return s + (e + q.y);
}
// accumulate w*x into the pair (h, l) for a pair weight (wh, wl) and a float x
__device__ __forceinline__ void ff_axpy(float wh, float wl, float x, float& h, float& l) {
  const float p = wh * x;
  const float pe = fmaf(wl, x, fmaf(wh, x, -p));  // exact error of wh*x, plus wl*x
  const float s = h + p;
  const float bb = s - h;
  const float e = (h - (s - bb)) + (p - bb);  // TwoSum error of h + p
  h = s;
  l = l + (e + pe);
}

template <bool INV, typename C>
__device__ __forceinline__ C cmul_mi(C a) { C r; if (INV) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r; }

// ---------------------------------------------------------------------------
// small DFTs, forward sign e^{-2 pi i pq/R}, inverse e^{+2 pi i pq/R}
// ---------------------------------------------------------------------------
template <typename T, bool INV>
__device__ __forceinline__ void dft2(cplx<T>* a) {
  cplx<T> t = a[0];
  a[0] = cadd(t, a[1]);
  a[1] = csub(t, a[1]);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4v(cplx<T>& a0, cplx<T>& a1, cplx<T>& a2, cplx<T>& a3) {
  cplx<T> t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = cmul_mi<INV>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(cplx<T>* a) { dft4v<T, INV>(a[0], a[1], a[2], a[3]); }

template <typename T, bool INV>
__device__ __forceinline__ void dft3(cplx<T>* a) {
  const T c = T(0.86602540378443864676372317075294);  // sqrt(3)/2
  cplx<T> s = cadd(a[1], a[2]), d = csub(a[1], a[2]);
  cplx<T> m = mkc<T>(a[0].x - T(0.5) * s.x, a[0].y - T(0.5) * s.y);
  a[0] = cadd(a[0], s);
  // (-i c) d forward, (+i c) d inverse
  cplx<T> r = cmul_mi<INV>(d);
  r.x *= c; r.y *= c;
  a[1] = cadd(m, r);
  a[2] = csub(m, r);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(cplx<T>* a) {
  const T h = T(0.70710678118654752440084436210485);  // 1/sqrt(2)
  cplx<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  cplx<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4v<T, INV>(e0, e1, e2, e3);
  dft4v<T, INV>(o0, o1, o2, o3);
  // twiddle the odd half by w8^q
  cplx<T> w1, w2, w3;
  if (!INV) {
    w1 = mkc<T>((o1.x + o1.y) * h, (o1.y - o1.x) * h);
    w2 = mkc<T>(o2.y, -o2.x);
    w3 = mkc<T>((o3.y - o3.x) * h, -(o3.x + o3.y) * h);
  } else {
    w1 = mkc<T>((o1.x - o1.y) * h, (o1.x + o1.y) * h);
    w2 = mkc<T>(-o2.y, o2.x);
    w3 = mkc<T>(-(o3.x + o3.y) * h, (o3.x - o3.y) * h);
  }
  a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
  a[1] = cadd(e1, w1); a[5] = csub(e1, w1);
  a[2] = cadd(e2, w2); a[6] = csub(e2, w2);
  a[3] = cadd(e3, w3); a[7] = csub(e3, w3);
}

__host__ __device__ constexpr int inv_mod(int a, int m) {
  for (int x = 1; x < m; ++x)
    if ((a * x) % m == 1) return x;
  return 1;
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dftR(cplx<T>* a);

// DFT of size R = R1 R2 with gcd(R1, R2) = 1 by the Good-Thomas prime-factor
// mapping: input n = (n1 R2 + n2 R1) mod R, output k = (k1 R2 u + k2 R1 v)
// mod R with u = R2^-1 mod R1, v = R1^-1 mod R2; a DFT-R1 over n1, then a
// DFT-R2 over n2, and no twiddle factors in between.  All indices are
// compile-time, so the permutations are register renamings.
template <typename T, bool INV, int R1, int R2>
__device__ __forceinline__ void dft_pfa(cplx<T>* a) {
  constexpr int R = R1 * R2;
  constexpr int U = inv_mod(R2, R1), V = inv_mod(R1, R2);
  cplx<T> t[R];
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2)
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) t[n2 * R1 + n1] = a[(n1 * R2 + n2 * R1) % R];
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) dftR<T, INV, R1>(&t[n2 * R1]);
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) {
    cplx<T> s[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) s[n2] = t[n2 * R1 + k1];
    dftR<T, INV, R2>(s);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) a[(k1 * R2 * U + k2 * R1 * V) % R] = s[k2];
  }
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dftR(cplx<T>* a) {
  if constexpr (R == 2) dft2<T, INV>(a);
  else if constexpr (R == 3) dft3<T, INV>(a);
  else if constexpr (R == 4) dft4<T, INV>(a);
  else if constexpr (R == 8) dft8<T, INV>(a);
  else if constexpr (R == 6) dft_pfa<T, INV, 2, 3>(a);
  else if constexpr (R == 12) dft_pfa<T, INV, 4, 3>(a);
  else static_assert(R == 2, "unsupported radix");
}

// ---------------------------------------------------------------------------
// compile-time plans: L -> radix list.  maxr >= 8: as many radix-8 stages as
// the power of two allows, the remaining factor 2 or 4 merged with one factor
// 3 into a radix-6 or radix-12 stage (when MF_FFT_COMPOSITE), then the other
// 3s; maxr 4: radix 4/2 stages, then 3s.  Merging keeps E = lcm(radices)
// unchanged and removes one shared-memory exchange.
// ---------------------------------------------------------------------------
#ifndef MF_FFT_COMPOSITE
#define MF_FFT_COMPOSITE 1
#endif
__host__ __device__ constexpr int ilog2_part(int L) { int a = 0; while (L % 2 == 0) { L /= 2; ++a; } return a; }
__host__ __device__ constexpr int i3_part(int L) { int b = 0; while (L % 3 == 0) { L /= 3; ++b; } return b; }
__host__ __device__ constexpr bool plan_ok(int L) {
  int x = L; while (x % 2 == 0) x /= 2; while (x % 3 == 0) x /= 3; return x == 1 && L >= 4;
}
struct FFTPlan {
  int n = 0;
  int r[16] = {};
};
__host__ __device__ constexpr FFTPlan make_plan(int L, int maxr) {
  FFTPlan p{};
  int a = ilog2_part(L), b = i3_part(L);
  if (maxr >= 8) {
    const int r8 = a / 3;
    int rem = a - 3 * r8;
    for (int i = 0; i < r8; ++i) p.r[p.n++] = 8;
    if (MF_FFT_COMPOSITE && rem > 0 && b > 0) {
      p.r[p.n++] = (rem == 1) ? 6 : 12;
      rem = 0;
      --b;
    }
    while (rem > 0) { const int t = (rem >= 2) ? 2 : 1; rem -= t; p.r[p.n++] = 1 << t; }
  } else {
    while (a > 0) { const int t = (a >= 2 && maxr >= 4) ? 2 : 1; a -= t; p.r[p.n++] = 1 << t; }
    if (MF_FFT_COMPOSITE && maxr >= 4 && b > 0 && p.n > 0 && p.r[p.n - 1] <= 4) {
      p.r[p.n - 1] *= 3;  // the last factor 4 or 2 merged with a factor 3 (radix 12 or 6)
      --b;
    }
  }
  for (int i = 0; i < b; ++i) p.r[p.n++] = 3;
  return p;
}
__host__ __device__ constexpr int plan_nstages(int L, int maxr) { return make_plan(L, maxr).n; }
__host__ __device__ constexpr int plan_radix(int L, int maxr, int s) {
  const FFTPlan p = make_plan(L, maxr);
  return (s < p.n) ? p.r[s] : 1;
}
__host__ __device__ constexpr int plan_elems(int L, int maxr) {
  // lcm of the radices
  int e = 1;
  for (int s = 0; s < plan_nstages(L, maxr); ++s) {
    int r = plan_radix(L, maxr, s);
    int g = e, h = r; while (h) { int t = g % h; g = h; h = t; }
    e = e / g * r;
  }
  return e;
}
__host__ __device__ constexpr int plan_lcur(int L, int maxr, int s) {
  int p = 1; for (int i = 0; i < s; ++i) p *= plan_radix(L, maxr, i); return p;
}

// Shared-memory layouts of the exchange buffer: element e of a line is kept
// at slot pidx<LAYOUT>(e) (times the element stride of the caller).
//   0  identity
//   1  one spare slot per 16 elements (e + e/16)
//   2  rows of a strided column tile: e ^ (bit 3 of e) in bit 0 -- with 8
//      columns of 8-byte elements per row this makes every exchange of the
//      radix-8-first plans take the minimum number of shared-memory
//      wavefronts (two 64-byte rows per half-warp land in different banks)
//   12, 13  XOR swizzles e ^ ((e >> s) & 15), s = 2 or 3, for contiguous
//      lines whose length is a multiple of 16 (a bijection on [0, L): only
//      the low four bits change, from higher bits)
// The layout of a contiguous-line exchange is picked per length (zlayout)
// from a count of shared-memory wavefronts per exchange instruction
// (16 lanes of 8-byte accesses per wavefront, 32 four-byte banks) over every
// write_out/read_in of the plan: the XOR swizzles reach the minimum for the
// radix-8-first plans of lengths 16..384 that are multiples of 16, where
// layout 1 takes up to twice as many for some exchanges.
template <int LAYOUT>
__device__ __forceinline__ int pidx(int e) {
  if constexpr (LAYOUT == 1) return e + (e >> 4);
  else if constexpr (LAYOUT == 2) return e ^ ((e >> 3) & 1);
  else if constexpr (LAYOUT == 12) return e ^ ((e >> 2) & 15);
  else if constexpr (LAYOUT == 13) return e ^ ((e >> 3) & 15);
  else return e;
}
__host__ __device__ constexpr int padded_len(int L, int layout) { return layout == 1 ? L + (L >> 4) + 1 : L; }
// exchange layout of a contiguous line of length L
__host__ __device__ constexpr int zlayout(int L) {
  return (L == 16 || L == 32 || L == 48 || L == 96 || L == 128 || L == 256 || L == 288 || L == 384 || L == 768)
             ? 13
             : ((L == 64 || L == 192) ? 12 : 1);
}
// distance between consecutive lines' exchange buffers (elements): the
// layout's length, widened where it moves the lines of one half-warp onto
// different banks
__host__ __device__ constexpr int zline_stride(int L) {
  switch (L) {
    case 16: return 18;
    case 24: return 27;
    case 32: return 36;
    case 48: return 50;
    case 64: return 65;
    case 96: return 100;
    case 144: return 155;
    case 192: return 193;
    case 288: return 292;
    default: return padded_len(L, zlayout(L)) | ((zlayout(L) == 1) ? 1 : 0);
  }
}

// Line FFT of length L in precision T, direction INV, radices up to MAXR;
// LAYOUT selects the shared-memory exchange index (pidx).  HOIST: a stage
// whose butterflies of one thread all share k = t mod LC (TPL a multiple of
// LC) loads its twiddles once instead of once per butterfly -- fewer L1
// loads, but the twiddles stay live across the butterflies, so it is for
// kernels with registers to spare (the strided passes at 128 registers
// spill with it).
template <typename T, int L, bool INV, int MAXR = 8, int LAYOUT = 0, bool HOIST = false>
struct LineFFT {
  static_assert(plan_ok(L), "FFT length must be 2^a 3^b >= 4");
  using C = cplx<T>;
  static constexpr int LEN = L;
  static constexpr int NS = plan_nstages(L, MAXR);
  static constexpr int E = plan_elems(L, MAXR);
  static constexpr int TPL = L / E;
  static constexpr int R0 = plan_radix(L, MAXR, 0);
  static constexpr int RL = plan_radix(L, MAXR, NS - 1);

  // stage-0 input element index of register slot (m*R0 + p)
  __device__ static __forceinline__ int in_index(int t, int slot) {
    return t + (slot / R0) * TPL + (slot % R0) * (L / R0);
  }
  // last-stage output element index of register slot (m*RL + q)
  __device__ static __forceinline__ int out_index(int t, int slot) {
    return t + (slot / RL) * TPL + (slot % RL) * (L / RL);
  }

  template <int S>
  __device__ static __forceinline__ void compute(C (&v)[E], int t, const C* __restrict__ tw) {
    constexpr int R = plan_radix(L, MAXR, S);
    constexpr int LC = plan_lcur(L, MAXR, S);
    constexpr int NB = E / R;
    if constexpr (HOIST && LC > 1 && TPL % LC == 0) {
      // every butterfly of this thread has the same k = t mod LC: one set of
      // twiddles for all of them
      constexpr int STR = L / (LC * R);
      const int k = t % LC;
      C w[R];
#pragma unroll
      for (int p = 1; p < R; ++p) w[p] = tw[p * k * STR];
#pragma unroll
      for (int m = 0; m < NB; ++m) {
#pragma unroll
        for (int p = 1; p < R; ++p) v[m * R + p] = INV ? cmulc(v[m * R + p], w[p]) : cmul(v[m * R + p], w[p]);
        dftR<T, INV, R>(&v[m * R]);
      }
      return;
    }
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      if constexpr (LC > 1) {
        const int b = t + m * TPL;
        const int k = b % LC;
        constexpr int STR = L / (LC * R);
#pragma unroll
        for (int p = 1; p < R; ++p) {
          const C w = tw[p * k * STR];
          v[m * R + p] = INV ? cmulc(v[m * R + p], w) : cmul(v[m * R + p], w);
        }
      }
      dftR<T, INV, R>(&v[m * R]);
    }
  }

  // write stage-S outputs to shared memory (element e at sm[e*cs])
  template <int S>
  __device__ static __forceinline__ void write_out(const C (&v)[E], int t, C* sm, int cs) {
    constexpr int R = plan_radix(L, MAXR, S);
    constexpr int LC = plan_lcur(L, MAXR, S);
    constexpr int NB = E / R;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      const int b = t + m * TPL;
      const int k = b % LC;
      const int base = (b - k) * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) sm[pidx<LAYOUT>(base + q * LC) * cs] = v[m * R + q];
    }
  }

  // read stage-S inputs from shared memory
  template <int S>
  __device__ static __forceinline__ void read_in(C (&v)[E], int t, const C* sm, int cs) {
    constexpr int R = plan_radix(L, MAXR, S);
    constexpr int NB = E / R;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      const int b = t + m * TPL;
#pragma unroll
      for (int p = 0; p < R; ++p) v[m * R + p] = sm[pidx<LAYOUT>(b + p * (L / R)) * cs];
    }
  }

  template <int S, class SYNC>
  __device__ static __forceinline__ void run_from(C (&v)[E], int t, C* sm, int cs, const C* __restrict__ tw, SYNC sync) {
    if constexpr (S < NS) {
      sync();
      write_out<S - 1>(v, t, sm, cs);
      sync();
      read_in<S>(v, t, sm, cs);
      compute<S>(v, t, tw);
      run_from<S + 1>(v, t, sm, cs, tw, sync);
    }
  }

  // v holds stage-0 inputs on entry and last-stage outputs on exit.  The
  // shared buffer (L elements at stride cs) may be overwritten; a sync is
  // issued before the first write, so callers may have read it just before.
  template <class SYNC>
  __device__ static __forceinline__ void run(C (&v)[E], int t, C* sm, int cs, const C* __restrict__ tw, SYNC sync) {
    compute<0>(v, t, tw);
    run_from<1>(v, t, sm, cs, tw, sync);
  }
};

struct SyncBlock { __device__ __forceinline__ void operator()() const { __syncthreads(); } };
// all lanes of a warp run the same line-group code path, so a full-mask
// warp barrier suffices when every line's threads sit inside one warp
struct SyncWarp { __device__ __forceinline__ void operator()() const { __syncwarp(); } };

}  // namespace mf
