// Kernel templates for the nLPT field pipeline: FFT passes with fused
// prologues/epilogues.  Data layout (same as Grid_FFT<real_t>, grid_fft.cc:45):
//   real space   [n0][n1][n2+2] reals, row-major (grid_fft.hh:184-188)
//   k space      [n0][n1][n2/2+1] complex, in place (grid_fft.hh:196-200)
// with i <-> kx, j <-> ky, k <-> kz >= 0 on a single device.
//
// Passes:
//   strided pass  (axis 0 or 1): one CTA owns NCOL consecutive kz columns of
//                 one slab; element e of column c lives at smem[e*NCOL + c],
//                 threads are column-fastest so every global row access is a
//                 contiguous NCOL*sizeof(complex) segment.
//   z pass        (axis 2): one thread group per line, lines contiguous in
//                 HBM; real transforms use the half-length complex packing.
#pragma once

#include "mf_fft.cuh"

namespace mf {

// ---------------------------------------------------------------------------
// strided column pass
// ---------------------------------------------------------------------------
// OP: __device__ C load(int slab, int e, int col) const;
//     __device__ void store(int slab, int e, int col, C v) const;
template <typename T, int L, bool INV, int NCOL, class OP>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, INV>::TPL)
k_colfft(OP op, const cplx<T>* __restrict__ tw, int ncols) {
  using F = LineFFT<T, L, INV>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int c = threadIdx.x, t = threadIdx.y;
  const int col = blockIdx.x * NCOL + c;
  const int slab = blockIdx.y;
  const bool valid = col < ncols;
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) {
    const int e = F::in_index(t, s);
    v[s] = valid ? op.load(slab, e, col) : mkc<T>(T(0), T(0));
  }
  F::run(v, t, sm + c, NCOL, tw, SyncBlock{});
  if (valid) {
#pragma unroll
    for (int s = 0; s < F::E; ++s) op.store(slab, F::out_index(t, s), col, v[s]);
  }
}

// ---------------------------------------------------------------------------
// z pass, real -> half complex (forward), one line per thread group
// OP: __device__ C load_pair(int line, int m) const;   // (x[2m], x[2m+1])
//     __device__ void store(int line, int k, C v) const;  // k in [0, kout)
// ---------------------------------------------------------------------------
template <typename T, int H, int NT, class OP>
__global__ void __launch_bounds__(NT) k_zr2c(OP op, const cplx<T>* __restrict__ twH,
                                               const cplx<T>* __restrict__ twM, int nlines, int kout) {
  using F = LineFFT<T, H, false>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * blockDim.y + ly;
  const bool valid = line < nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * (H + 1);
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) v[s] = valid ? op.load_pair(line, F::in_index(t, s)) : mkc<T>(T(0), T(0));
  F::run(v, t, sm, 1, twH, SyncBlock{});
  __syncthreads();
#pragma unroll
  for (int s = 0; s < F::E; ++s) sm[F::out_index(t, s)] = v[s];
  __syncthreads();
  if (valid) {
    for (int k = t; k < kout; k += F::TPL) {
      const C zk = sm[k % H];
      const C zc = cconj(sm[(H - k) % H]);
      const C E = mkc<T>(T(0.5) * (zk.x + zc.x), T(0.5) * (zk.y + zc.y));
      // O = (zk - zc) / (2i)
      const C O = mkc<T>(T(0.5) * (zk.y - zc.y), -T(0.5) * (zk.x - zc.x));
      op.store(line, k, cadd(E, cmul(twM[k], O)));
    }
  }
}

// ---------------------------------------------------------------------------
// z pass, half complex -> real (inverse), Re-semantics of FFTW's c2r
// OP: __device__ C load(int line, int k) const;          // k in [0, H]
//     __device__ void store_pair(int line, int m, C v) const;
// ---------------------------------------------------------------------------
template <typename T, int H>
__device__ __forceinline__ cplx<T> c2r_pre(const cplx<T>* sm, int k, const cplx<T>* __restrict__ twM) {
  using C = cplx<T>;
  C A = sm[k];
  C B = cconj(sm[H - k]);
  if (k == 0) { A.y = T(0); B.y = T(0); }
  const C Ev = cadd(A, B);
  const C Ov = cmulc(csub(A, B), twM[k]);  // (A-B) e^{+2 pi i k/M}
  return mkc<T>(Ev.x - Ov.y, Ev.y + Ov.x);  // E + i O
}

template <typename T, int H, int NT, class OP>
__global__ void __launch_bounds__(NT) k_zc2r(OP op, const cplx<T>* __restrict__ twH,
                                               const cplx<T>* __restrict__ twM, int nlines, int kin) {
  using F = LineFFT<T, H, true>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * blockDim.y + ly;
  const bool valid = line < nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * (H + 1);
  for (int k = t; k <= H; k += F::TPL) sm[k] = (valid && k < kin) ? op.load(line, k) : mkc<T>(T(0), T(0));
  __syncthreads();
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) v[s] = c2r_pre<T, H>(sm, F::in_index(t, s), twM);
  F::run(v, t, sm, 1, twH, SyncBlock{});
  if (valid) {
#pragma unroll
    for (int s = 0; s < F::E; ++s) op.store_pair(line, F::out_index(t, s), v[s]);
  }
}

// ---------------------------------------------------------------------------
// fused Orszag z pass: per line, c2r of nop operands, pointwise product of
// the real values, r2c of the product, store of kz in [0, kout)
// ---------------------------------------------------------------------------

template <typename T, int H, int NT>
__global__ void __launch_bounds__(NT) k_zconv(ZConvArgs<T> a, const cplx<T>* __restrict__ twH,
                                                const cplx<T>* __restrict__ twM) {
  using FI = LineFFT<T, H, true>;
  using FF = LineFFT<T, H, false>;
  static_assert(FI::E == FF::E && FI::TPL == FF::TPL, "plan mismatch");
  using C = cplx<T>;
  constexpr int E = FI::E, TPL = FI::TPL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * blockDim.y + ly;
  const bool valid = line < a.nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * (2 * H + 2);
  C* prod = sm + (H + 1);  // per-thread-owned slots of the running product
  C v[E];
  for (int op = 0; op < a.nop; ++op) {
    __syncthreads();
    const C* src = a.in[op] + (long long)line * a.in_stride;
    for (int k = t; k <= H; k += TPL) sm[k] = (valid && k < a.kin) ? src[k] : mkc<T>(T(0), T(0));
    __syncthreads();
#pragma unroll
    for (int s = 0; s < E; ++s) v[s] = c2r_pre<T, H>(sm, FI::in_index(t, s), twM);
    FI::run(v, t, sm, 1, twH, SyncBlock{});
    // v[s] = (x[2m], x[2m+1]) with m = out_index(t, s); slots are thread-owned
#pragma unroll
    for (int s = 0; s < E; ++s) {
      const int m = FI::out_index(t, s);
      if (op == 0) prod[m] = v[s];
      else { C p = prod[m]; p.x *= v[s].x; p.y *= v[s].y; prod[m] = p; }
    }
  }
  __syncthreads();
  // forward transform of the packed product
#pragma unroll
  for (int s = 0; s < E; ++s) v[s] = prod[FF::in_index(t, s)];
  FF::run(v, t, sm, 1, twH, SyncBlock{});
  __syncthreads();
#pragma unroll
  for (int s = 0; s < E; ++s) sm[FF::out_index(t, s)] = v[s];
  __syncthreads();
  if (valid) {
    C* dst = a.out + (long long)line * a.out_stride;
    for (int k = t; k < a.kout; k += TPL) {
      const C zk = sm[k % H];
      const C zc = cconj(sm[(H - k) % H]);
      const C Ev = mkc<T>(T(0.5) * (zk.x + zc.x), T(0.5) * (zk.y + zc.y));
      const C Ov = mkc<T>(T(0.5) * (zk.y - zc.y), -T(0.5) * (zk.x - zc.x));
      dst[k] = cscale(cadd(Ev, cmul(twM[k], Ov)), a.out_scale);
    }
  }
}

}  // namespace mf
