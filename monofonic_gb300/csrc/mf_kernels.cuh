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

#include <type_traits>

#include "mf_fft.cuh"
#include "mf_tma.cuh"

// largest radix of the pipelined strided passes' plans (a build-time knob)
#ifndef MF_COL_MAXR
#define MF_COL_MAXR 8
#endif
// threads per CTA up to which the pipelined strided passes are compiled for two
// resident CTAs per SM (a register cap of 65536 / (2 x threads)); a build-time knob.
// 512 puts two 512-thread CTAs of the FP32 length-512 passes on an SM (64
// registers, no spills): 0.4 ms less per 512^3 3LPT IC than one CTA at 256.
#ifndef MF_COL_MINB_LIMIT
#define MF_COL_MINB_LIMIT 512
#endif
// 1: the pipelined strided passes' resident CTAs per SM sized from the
// registers the plan needs (~4 per scalar held, plus 32) instead of the rule
// above, at most 4; a build-time knob.  The 128-thread CTAs of the FP32
// length-96..384 passes were compiled for two CTAs per SM and took up to 255
// registers (8 warps per SM); sized for four (128 registers, no spills) the
// N=256 3LPT IC takes 10.9 instead of 11.7 ms and the 96-realization batch
// 215 instead of 231 ms.  M=768 and N=512 passes compile as before.
#ifndef MF_COL_REG_SIZED
#define MF_COL_REG_SIZED 1
#endif

namespace mf {

// minimum resident CTAs per SM a pipelined strided pass is compiled for
// (its __launch_bounds__): threads per CTA, values per thread E of the plan,
// bytes per scalar
__host__ __device__ constexpr int col_minb(int threads, int e, int scalar_bytes) {
  if (!MF_COL_REG_SIZED) return threads <= MF_COL_MINB_LIMIT ? 2 : 1;
  int need = 4 * e * (scalar_bytes / 4) + 32;
  need = need < 64 ? 64 : (need > 255 ? 255 : need);
  const int b = 65536 / (threads * need);
  return b < 1 ? 1 : (b > 4 ? 4 : b);
}

// exchange layout of a pipelined strided tile [row e][NCOL columns]: the
// row swizzle (pidx<2>) where a row is 64 bytes (8 FP32 or 4 FP64 complex
// columns) and the op asks for it (kColSwizzle), identity otherwise.  The
// swizzle's per-element address arithmetic costs registers: the ops with a
// prologue or a prefetched read-modify-write target (x passes) sit at the
// 128-register cap of two CTAs per SM and would spill, so they keep the
// identity layout.
template <class OP, class = void>
struct col_swizzle : std::false_type {};
template <class OP>
struct col_swizzle<OP, std::void_t<decltype(OP::kColSwizzle)>> : std::integral_constant<bool, OP::kColSwizzle> {};
template <typename T, int NCOL, class OP>
__host__ __device__ constexpr int col_layout() {
  return (col_swizzle<OP>::value && NCOL * (int)sizeof(cplx<T>) == 64) ? 2 : 0;
}

// ops with a per-tile prologue (tile_prep / xform_tile) in the pipelined pass
template <class OP, class = void>
struct has_tile_prep : std::false_type {};
template <class OP>
struct has_tile_prep<OP, std::void_t<decltype(&OP::tile_prep)>> : std::true_type {};

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
  if constexpr (OP::kPrefetch) {
    C pre[F::E];
#pragma unroll
    for (int s = 0; s < F::E; ++s) pre[s] = valid ? op.prefetch(slab, F::out_index(t, s), col) : mkc<T>(T(0), T(0));
    F::run(v, t, sm + c, NCOL, tw, SyncBlock{});
    if (valid) {
#pragma unroll
      for (int s = 0; s < F::E; ++s) op.store_pre(slab, F::out_index(t, s), col, v[s], pre[s]);
    }
  } else {
    F::run(v, t, sm + c, NCOL, tw, SyncBlock{});
    if (valid) {
#pragma unroll
      for (int s = 0; s < F::E; ++s) op.store(slab, F::out_index(t, s), col, v[s]);
    }
  }
}

// strided pass producing three transforms per column (three-component
// assembly): the loader yields the three inputs of each element at once, the
// three line FFTs run one after the other through the same shared tile
template <typename T, int L, bool INV, int NCOL, class OP>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, INV>::TPL)
k_colfft3(OP op, const cplx<T>* __restrict__ tw, int ncols) {
  using F = LineFFT<T, L, INV>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int c = threadIdx.x, t = threadIdx.y;
  const int col = blockIdx.x * NCOL + c;
  const int slab = blockIdx.y;
  const bool valid = col < ncols;
  C v[3][F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) {
    C w[3] = {mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0))};
    if (valid) op.load3(slab, F::in_index(t, s), col, w);
    v[0][s] = w[0];
    v[1][s] = w[1];
    v[2][s] = w[2];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    F::run(v[d], t, sm + c, NCOL, tw, SyncBlock{});
    if (valid) {
#pragma unroll
      for (int s = 0; s < F::E; ++s) op.store(d, slab, F::out_index(t, s), col, v[d][s]);
    }
  }
}

// The same staged through shared memory: the first component stays in
// registers, the other two go to their own tiles as they are loaded, and each
// later component's transform runs from (and exchanges through) its tile, so
// registers hold one component and two CTAs share an SM (one's loads overlap
// the other's transforms).  Every thread reads back only the tile slots it
// wrote (the first stage's inputs), so no barrier precedes the reads.
template <typename T, int L, bool INV, int NCOL, class OP, int MINB>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, INV>::TPL, MINB)
k_colfft3s(OP op, const cplx<T>* __restrict__ tw, int ncols) {
  using F = LineFFT<T, L, INV>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* xchg = reinterpret_cast<C*>(smem_raw);  // exchanges of the first component
  C* tile1 = xchg + L * NCOL;
  C* tile2 = tile1 + L * NCOL;
  const int c = threadIdx.x, t = threadIdx.y;
  const int col = blockIdx.x * NCOL + c;
  const int slab = blockIdx.y;
  const bool valid = col < ncols;
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) {
    const int e = F::in_index(t, s);
    C w[3] = {mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0)), mkc<T>(T(0), T(0))};
    if (valid) op.load3(slab, e, col, w);
    v[s] = w[0];
    tile1[e * NCOL + c] = w[1];
    tile2[e * NCOL + c] = w[2];
  }
  F::run(v, t, xchg + c, NCOL, tw, SyncBlock{});
  if (valid) {
#pragma unroll
    for (int s = 0; s < F::E; ++s) op.store(0, slab, F::out_index(t, s), col, v[s]);
  }
#pragma unroll
  for (int d = 1; d < 3; ++d) {
    C* tl = (d == 1) ? tile1 : tile2;
#pragma unroll
    for (int s = 0; s < F::E; ++s) v[s] = tl[F::in_index(t, s) * NCOL + c];
    F::run(v, t, tl + c, NCOL, tw, SyncBlock{});
    if (valid) {
#pragma unroll
      for (int s = 0; s < F::E; ++s) op.store(d, slab, F::out_index(t, s), col, v[s]);
    }
  }
}

// ---------------------------------------------------------------------------
// persistent, double-buffered strided pass.  Each CTA walks tiles
// (column tile, slab, operand) with stride gridDim.x; while a tile is being
// transformed, the raw elements of the CTA's next tile are already being
// copied into the other shared-memory buffer with cp.async.  Every thread
// copies exactly the elements it reads for its first FFT stage, so a
// per-thread wait_group suffices before the read.
// OP: kPipe, srcp(z, slab, e, col) -> const C* (nullptr = zero),
//     xform(z, slab, e, col, raw), store_z(z, slab, e, col, v)
//     (+ kPrefetch: prefetch/store_pre on the same coordinates)
// ---------------------------------------------------------------------------
template <typename T, int L, bool INV, int NCOL, class OP>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, INV, MF_COL_MAXR>::TPL,
                                  col_minb(NCOL * LineFFT<T, L, INV, MF_COL_MAXR>::TPL,
                                           LineFFT<T, L, INV, MF_COL_MAXR>::E, (int)sizeof(T)))
k_colfft_pipe(OP op, const cplx<T>* __restrict__ tw, int ncols, int ntc, int nslab, int nz) {
  constexpr int LAY = col_layout<T, NCOL, OP>();
  using F = LineFFT<T, L, INV, MF_COL_MAXR, LAY>;
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + L * NCOL;
  const int c = threadIdx.x, t = threadIdx.y;
  const int total = ntc * nslab * nz;
  auto issue = [&](int tl, C* buf) {
    const int ct = tl % ntc, r = tl / ntc, slab = r % nslab, z = r / nslab;
    const int col = ct * NCOL + c;
#pragma unroll
    for (int s = 0; s < F::E; ++s) {
      const int e = F::in_index(t, s);
      C* d = buf + pidx<LAY>(e) * NCOL + c;
      const C* g = (col < ncols) ? op.srcp(z, slab, e, col) : nullptr;
      if (g) {
        if constexpr (sizeof(C) == 16) cp_async16(d, g); else cp_async8(d, g);
      } else {
        *d = mkc<T>(T(0), T(0));
      }
    }
    cp_async_commit();
  };
  int tl = blockIdx.x;
  if (tl < total) issue(tl, buf0); else cp_async_commit();
  for (int it = 0; tl < total; tl += gridDim.x, ++it) {
    C* cur = (it & 1) ? buf1 : buf0;
    C* nxt = (it & 1) ? buf0 : buf1;
    const int tn = tl + gridDim.x;
    if (tn < total) issue(tn, nxt); else cp_async_commit();
    cp_async_wait<1>();
    const int ct = tl % ntc, r = tl / ntc, slab = r % nslab, z = r / nslab;
    const int col = ct * NCOL + c;
    const bool valid = col < ncols;
    C v[F::E];
    if constexpr (has_tile_prep<OP>::value) {
      const auto tp = op.tile_prep(z, slab, col);
#pragma unroll
      for (int s = 0; s < F::E; ++s) {
        const int e = F::in_index(t, s);
        v[s] = valid ? op.xform_tile(tp, e, cur[pidx<LAY>(e) * NCOL + c]) : mkc<T>(T(0), T(0));
      }
    } else {
#pragma unroll
      for (int s = 0; s < F::E; ++s) {
        const int e = F::in_index(t, s);
        v[s] = valid ? op.xform(z, slab, e, col, cur[pidx<LAY>(e) * NCOL + c]) : mkc<T>(T(0), T(0));
      }
    }
    if constexpr (OP::kPrefetch) {
      C pre[F::E];
#pragma unroll
      for (int s = 0; s < F::E; ++s) pre[s] = valid ? op.prefetch(slab, F::out_index(t, s), col) : mkc<T>(T(0), T(0));
      F::run(v, t, cur + c, NCOL, tw, SyncBlock{});
      if (valid) {
#pragma unroll
        for (int s = 0; s < F::E; ++s) op.store_pre(slab, F::out_index(t, s), col, v[s], pre[s]);
      }
    } else {
      F::run(v, t, cur + c, NCOL, tw, SyncBlock{});
      if (valid) {
#pragma unroll
        for (int s = 0; s < F::E; ++s) op.store_z(z, slab, F::out_index(t, s), col, v[s]);
      }
    }
    __syncthreads();  // cur is refilled by the next iteration's copies
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// The same pass with one column per line group inside a warp (a build-time
// variant, MF_COL_WPC): the tile is staged column-major ([column][row], column
// stride LSC = 4 mod 16 elements, so the row-major staging copies and the
// copy-out reads take the minimum number of wavefronts), each column's
// transform exchanges through its own column under warp barriers (the XOR
// layout of the contiguous-line passes), and the results go back to global
// memory in 64-byte row runs from a column-major copy-out.  Ops with a
// prefetched read-modify-write target are not eligible.
// ---------------------------------------------------------------------------
template <typename T, int L, bool INV>
__host__ __device__ constexpr int wpc_lsc() {
  constexpr int base = padded_len(L, zlayout(L));
  return base + ((4 - base % 16) % 16 + 16) % 16;
}
template <typename T, int L, bool INV, class OP>
__host__ __device__ constexpr bool wpc_ok() {
  using F = LineFFT<T, L, INV, MF_COL_MAXR>;
  return !OP::kPrefetch && F::TPL <= 32 && 32 % F::TPL == 0;
}
template <typename T, int L, bool INV, int NCOL, class OP>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, INV, MF_COL_MAXR>::TPL,
                                  col_minb(NCOL * LineFFT<T, L, INV, MF_COL_MAXR>::TPL,
                                           LineFFT<T, L, INV, MF_COL_MAXR>::E, (int)sizeof(T)))
k_colfft_wpc(OP op, const cplx<T>* __restrict__ tw, int ncols, int ntc, int nslab, int nz) {
  using F = LineFFT<T, L, INV, MF_COL_MAXR, zlayout(L)>;
  using C = cplx<T>;
  constexpr int LSC = wpc_lsc<T, L, INV>();
  constexpr int NT = NCOL * F::TPL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + NCOL * LSC;
  const int tid = threadIdx.x;
  const int cl = tid / F::TPL, t = tid % F::TPL;  // this thread's column in the tile and its line slot
  const int total = ntc * nslab * nz;
  auto issue = [&](int tl, C* buf) {
    const int ct = tl % ntc, r = tl / ntc, slab = r % nslab, z = r / nslab;
#pragma unroll 4
    for (int u = tid; u < L * NCOL; u += NT) {
      const int e = u / NCOL, c = u % NCOL;
      const int col = ct * NCOL + c;
      C* d = buf + c * LSC + e;
      const C* g = (col < ncols) ? op.srcp(z, slab, e, col) : nullptr;
      if (g) {
        if constexpr (sizeof(C) == 16) cp_async16(d, g); else cp_async8(d, g);
      } else {
        *d = mkc<T>(T(0), T(0));
      }
    }
    cp_async_commit();
  };
  int tl = blockIdx.x;
  if (tl < total) issue(tl, buf0); else cp_async_commit();
  for (int it = 0; tl < total; tl += gridDim.x, ++it) {
    C* cur = (it & 1) ? buf1 : buf0;
    C* nxt = (it & 1) ? buf0 : buf1;
    const int tn = tl + gridDim.x;
    if (tn < total) issue(tn, nxt); else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();  // every thread's copies of this tile have landed
    const int ct = tl % ntc, r = tl / ntc, slab = r % nslab, z = r / nslab;
    const int col = ct * NCOL + cl;
    const bool valid = col < ncols;
    C* cb = cur + cl * LSC;
    C v[F::E];
    if constexpr (has_tile_prep<OP>::value) {
      const auto tp = op.tile_prep(z, slab, col);
#pragma unroll
      for (int s = 0; s < F::E; ++s) {
        const int e = F::in_index(t, s);
        v[s] = valid ? op.xform_tile(tp, e, cb[e]) : mkc<T>(T(0), T(0));
      }
    } else {
#pragma unroll
      for (int s = 0; s < F::E; ++s) {
        const int e = F::in_index(t, s);
        v[s] = valid ? op.xform(z, slab, e, col, cb[e]) : mkc<T>(T(0), T(0));
      }
    }
    F::run(v, t, cb, 1, tw, SyncWarp{});
    __syncwarp();  // the column's last exchange has been read
#pragma unroll
    for (int s = 0; s < F::E; ++s) cb[F::out_index(t, s)] = v[s];
    __syncthreads();  // every column of the tile is transformed
#pragma unroll 4
    for (int u = tid; u < L * NCOL; u += NT) {
      const int e = u / NCOL, c = u % NCOL;
      const int cc = ct * NCOL + c;
      if (cc < ncols) op.store_z(z, slab, e, cc, cur[c * LSC + e]);
    }
    __syncthreads();  // cur is refilled by the next iteration's copies
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// strided forward transform, truncation and inverse transform of one column in
// one pass (ConvXTruncOp), persistent and double-buffered as k_colfft_pipe
// ---------------------------------------------------------------------------
template <typename T, int L, int NCOL, class OP>
__global__ void __launch_bounds__(NCOL * LineFFT<T, L, false, MF_COL_MAXR>::TPL,
                                  col_minb(NCOL * LineFFT<T, L, false, MF_COL_MAXR>::TPL,
                                           LineFFT<T, L, false, MF_COL_MAXR>::E, (int)sizeof(T)))
k_colfft_trunc(OP op, const cplx<T>* __restrict__ tw, int ncols, int ntc, int nslab) {
  constexpr int LAY = col_layout<T, NCOL, OP>();
  using FF = LineFFT<T, L, false, MF_COL_MAXR, LAY>;
  using FI = LineFFT<T, L, true, MF_COL_MAXR, LAY>;
  static_assert(FF::E == FI::E && FF::TPL == FI::TPL, "one plan for both directions");
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + L * NCOL;
  const int c = threadIdx.x, t = threadIdx.y;
  const int total = ntc * nslab;
  auto issue = [&](int tl, C* buf) {
    const int ct = tl % ntc, slab = tl / ntc;
    const int col = ct * NCOL + c;
#pragma unroll
    for (int s = 0; s < FF::E; ++s) {
      const int e = FF::in_index(t, s);
      C* d = buf + pidx<LAY>(e) * NCOL + c;
      if (col < ncols) {
        if constexpr (sizeof(C) == 16) cp_async16(d, op.at(slab, e, col)); else cp_async8(d, op.at(slab, e, col));
      } else {
        *d = mkc<T>(T(0), T(0));
      }
    }
    cp_async_commit();
  };
  int tl = blockIdx.x;
  if (tl < total) issue(tl, buf0); else cp_async_commit();
  for (int it = 0; tl < total; tl += gridDim.x, ++it) {
    C* cur = (it & 1) ? buf1 : buf0;
    C* nxt = (it & 1) ? buf0 : buf1;
    const int tn = tl + gridDim.x;
    if (tn < total) issue(tn, nxt); else cp_async_commit();
    cp_async_wait<1>();
    const int ct = tl % ntc, slab = tl / ntc;
    const int col = ct * NCOL + c;
    const bool valid = col < ncols;
    C v[FF::E];
#pragma unroll
    for (int s = 0; s < FF::E; ++s) v[s] = cur[pidx<LAY>(FF::in_index(t, s)) * NCOL + c];
    FF::run(v, t, cur + c, NCOL, tw, SyncBlock{});
    __syncthreads();  // the last exchange of the forward transform has been read
#pragma unroll
    for (int s = 0; s < FF::E; ++s) {
      const int e = FF::out_index(t, s);
      cur[pidx<LAY>(e) * NCOL + c] = op.mask(slab, e, col, v[s]);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < FI::E; ++s) v[s] = cur[pidx<LAY>(FI::in_index(t, s)) * NCOL + c];
    FI::run(v, t, cur + c, NCOL, tw, SyncBlock{});
    if (valid) {
#pragma unroll
      for (int s = 0; s < FI::E; ++s) *op.at(slab, FI::out_index(t, s), col) = v[s];
    }
    __syncthreads();  // cur is refilled by the next iteration's copies
  }
  cp_async_wait<0>();
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
  // a line's shared-memory area is its own: warp barriers when its threads sit inside one warp
  using SYNC = typename std::conditional<(F::TPL <= 32 && 32 % F::TPL == 0 && NT % 32 == 0), SyncWarp, SyncBlock>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * blockDim.y + ly;
  const bool valid = line < nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * (H + 1);
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) v[s] = valid ? op.load_pair(line, F::in_index(t, s)) : mkc<T>(T(0), T(0));
  F::run(v, t, sm, 1, twH, SYNC{});
  SYNC{}();
#pragma unroll
  for (int s = 0; s < F::E; ++s) sm[F::out_index(t, s)] = v[s];
  SYNC{}();
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
  // a line's shared-memory area is its own: warp barriers when its threads sit inside one warp
  using SYNC = typename std::conditional<(F::TPL <= 32 && 32 % F::TPL == 0 && NT % 32 == 0), SyncWarp, SyncBlock>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * blockDim.y + ly;
  const bool valid = line < nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * (H + 1);
  for (int k = t; k <= H; k += F::TPL) sm[k] = (valid && k < kin) ? op.load(line, k) : mkc<T>(T(0), T(0));
  SYNC{}();
  C v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) v[s] = c2r_pre<T, H>(sm, F::in_index(t, s), twM);
  F::run(v, t, sm, 1, twH, SYNC{});
  if (valid) {
#pragma unroll
    for (int s = 0; s < F::E; ++s) op.store_pair(line, F::out_index(t, s), v[s]);
  }
}

// ---------------------------------------------------------------------------
// z pass c2r of the three displacement / velocity components of a line, with
// the lattice readout fused (set_positions / set_velocities,
// particle_generator.hh:499-639): particle ip = ishift*n^3 + cell, AoS
// [ip][3] of q + Psi (FP64 sum, stored as P) or, in fields mode, three n^3
// grids of doubles.  Inputs: the three component grids after their x and y
// passes, [line][n/2+1] complex.
// ---------------------------------------------------------------------------
// the lattice readout of one transformed line (particle ip = ishift*n^3 + cell)
template <typename T, int H, typename P>
__device__ __forceinline__ void lattice_line_out(Lattice3Args a, int line, int t,
                                                 const cplx<T> (&v)[3][LineFFT<T, H, true>::E]) {
  using F = LineFFT<T, H, true>;
  const int n = a.n;
  const long long n3 = (long long)n * n * n;
  const int i = line / n, j = line % n;
  if constexpr (std::is_same<P, float>::value && std::is_same<T, float>::value) {
    if (!a.fields_mode) {
      // FP32 particles: the two particles 2m, 2m+1 of a slot are 24 contiguous
      // bytes (8-byte aligned for even n), stored as three float2
#pragma unroll
      for (int s = 0; s < F::E; ++s) {
        const int m = F::out_index(t, s);
        float w[6];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int k = 2 * m + h;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float x = (h ? v[d][s].y : v[d][s].x) * T(a.norm);
            const int qi = (d == 0) ? i : ((d == 1) ? n + j : 2 * n + k);
            w[3 * h + d] = a.with_q ? ff_add_q(a.qf[qi], x) : x;
          }
        }
        float2* o = reinterpret_cast<float2*>(reinterpret_cast<float*>(a.dst) +
                                              3 * ((long long)a.ishift * n3 + (long long)line * n + 2 * m));
        o[0] = make_float2(w[0], w[1]);
        o[1] = make_float2(w[2], w[3]);
        o[2] = make_float2(w[4], w[5]);
      }
      return;
    }
  }
#pragma unroll
  for (int s = 0; s < F::E; ++s) {
    const int m = F::out_index(t, s);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 2 * m + h;
      const long long c = (long long)line * n + k;
      if (std::is_same<P, T>::value && !a.with_q && !a.fields_mode) {
        // velocities (no lattice coordinate) in the grid precision: no FP64 step
        P* o = reinterpret_cast<P*>(a.dst) + 3 * ((long long)a.ishift * n3 + c);
#pragma unroll
        for (int d = 0; d < 3; ++d) o[d] = (P)((h ? v[d][s].y : v[d][s].x) * T(a.norm));
        continue;
      }
      if constexpr (std::is_same<P, float>::value && std::is_same<T, float>::value) {
        if (a.with_q && !a.fields_mode) {
          // FP32 positions q + Psi with q as a float pair: the correctly
          // rounded sum on the FP32 pipes (ff_add_q)
          P* o = reinterpret_cast<P*>(a.dst) + 3 * ((long long)a.ishift * n3 + c);
          const int qi[3] = {i, n + j, 2 * n + k};
#pragma unroll
          for (int d = 0; d < 3; ++d) o[d] = ff_add_q(a.qf[qi[d]], (h ? v[d][s].y : v[d][s].x) * T(a.norm));
          continue;
        }
      }
      double val[3];
      // normalised in the grid precision, as the component grids of the per-component path
#pragma unroll
      for (int d = 0; d < 3; ++d) val[d] = (double)((h ? v[d][s].y : v[d][s].x) * T(a.norm));
      if (a.fields_mode) {
        double* o = reinterpret_cast<double*>(a.dst);
#pragma unroll
        for (int d = 0; d < 3; ++d) o[d * n3 + c] = val[d];
      } else {
        if (a.with_q) {
          val[0] += a.q[i];
          val[1] += a.q[n + j];
          val[2] += a.q[2 * n + k];
        }
        P* o = reinterpret_cast<P*>(a.dst) + 3 * ((long long)a.ishift * n3 + c);
#pragma unroll
        for (int d = 0; d < 3; ++d) o[d] = (P)val[d];
      }
    }
  }
}


template <typename T, int H, int LPB, typename P>
__global__ void __launch_bounds__(LPB * LineFFT<T, H, true>::TPL, (LineFFT<T, H, true>::E <= 8) ? 2 : 1)
    k_zc2r3_lattice(Lattice3Args a, const cplx<T>* __restrict__ twH, const cplx<T>* __restrict__ twM) {
  // each line's exchanges run in its own staged region (XOR layout of the
  // contiguous-line passes), under warp barriers when a line's threads sit
  // inside one warp
  // (the identity layout where three components of E > 8 values already fill the registers)
  using F = LineFFT<T, H, true, 8, (LineFFT<T, H, true>::E <= 8) ? zlayout(H) : 0>;
  using SYNC = typename std::conditional<(F::TPL <= 32 && 32 % F::TPL == 0 && (LPB * F::TPL) % 32 == 0), SyncWarp,
                                         SyncBlock>::type;
  using C = cplx<T>;
  constexpr int SL = 3 * (H + 1);  // complex values of one line's three components
  // persistent CTAs over batches of LPB lines; the next batch is copied into
  // the other shared-memory buffer (cp.async) while this one is transformed
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  C* buf1 = buf0 + LPB * SL;
  const int t = threadIdx.x, ly = threadIdx.y;
  const int tid = ly * F::TPL + t;
  const int n = a.n, Kz = H + 1;
  const int nb = (a.nlines + LPB - 1) / LPB;
  // a batch of one component is LPB consecutive lines, contiguous in global
  // memory: staged as [d][l][k] with 16-byte copies (an even LPB keeps both
  // ends 16-byte aligned)
  static_assert(LPB % 2 == 0, "even lines per batch");
  constexpr int U = LPB * Kz * (int)sizeof(C) / 16;  // 16-byte units per component
  auto issue = [&](int bt, C* buf) {  // nlines is a multiple of LPB (checked at launch)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const void* base = (d == 0) ? a.comp[0] : ((d == 1) ? a.comp[1] : a.comp[2]);
      const char* g = reinterpret_cast<const char*>(base) + (size_t)bt * LPB * Kz * sizeof(C);
      char* sb = reinterpret_cast<char*>(buf + d * LPB * Kz);
      for (int u = tid; u < U; u += LPB * F::TPL) cp_async16(sb + 16 * u, g + 16 * u);
    }
    cp_async_commit();
  };
  int bt = blockIdx.x;
  if (bt < nb) issue(bt, buf0); else cp_async_commit();
  for (int it = 0; bt < nb; bt += gridDim.x, ++it) {
    C* cur = (it & 1) ? buf1 : buf0;
    C* nxt = (it & 1) ? buf0 : buf1;
    const int bn = bt + gridDim.x;
    if (bn < nb) issue(bn, nxt); else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();  // every thread's copies of this batch have landed
    const int line = bt * LPB + ly;
    const bool valid = line < a.nlines;
    C* sm[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) sm[d] = cur + d * LPB * Kz + ly * Kz;
    C v[3][F::E];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int s = 0; s < F::E; ++s) v[d][s] = c2r_pre<T, H>(sm[d], F::in_index(t, s), twM);
#pragma unroll
    for (int d = 0; d < 3; ++d) F::run(v[d], t, sm[d], 1, twH, SYNC{});
    if (valid) lattice_line_out<T, H, P>(a, line, t, v);
    __syncthreads();  // cur is refilled by the next iteration's copies
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// fused Orszag z pass: per line, c2r of nop operands, pointwise product of
// the real values, r2c of the product, store of kz in [0, kout)
// ---------------------------------------------------------------------------

// c2r pre-processing read straight from global memory: Z[k] = E + i O with
// A = X[k], B = conj(X[H-k]) (zero for kz >= kin), imaginary parts of the
// kz = 0 and kz = H terms dropped (FFTW's c2r convention)
template <typename T, int H>
__device__ __forceinline__ cplx<T> c2r_pre_g(const cplx<T>* __restrict__ src, int k, int kin,
                                             const cplx<T>* __restrict__ twM) {
  using C = cplx<T>;
  C A = (k < kin) ? src[k] : mkc<T>(T(0), T(0));
  C B = (H - k < kin) ? src[H - k] : mkc<T>(T(0), T(0));
  if (k == 0) { A.y = T(0); B.y = T(0); }
  B = cconj(B);
  const C Ev = cadd(A, B);
  const C Ov = cmulc(csub(A, B), twM[k]);
  return mkc<T>(Ev.x - Ov.y, Ev.y + Ov.x);
}

// One thread group of TPL threads per line; when TPL divides 32 every line
// lives inside one warp and all exchanges use warp barriers only.  The
// operands' inverse transforms read their inputs straight from HBM, the
// running product stays in registers, and only the final r2c
// post-processing goes through shared memory once more.
template <typename T, int H, int MAXR, int NT, int MINB, class SYNC>
__global__ void __launch_bounds__(NT, MINB) k_zconv(ZConvArgs<T> a, const cplx<T>* __restrict__ twH,
                                                const cplx<T>* __restrict__ twM) {
  using FI = LineFFT<T, H, true, MAXR>;
  using FF = LineFFT<T, H, false, MAXR>;
  static_assert(FI::E == FF::E && FI::TPL == FF::TPL, "plan mismatch");
  using C = cplx<T>;
  constexpr int E = FI::E, TPL = FI::TPL, LPB = NT / TPL;
  constexpr int LSTRIDE = H + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x % TPL, ly = threadIdx.x / TPL;
  const int line = blockIdx.x * LPB + ly;
  const bool valid = line < a.nlines;
  C* sm = reinterpret_cast<C*>(smem_raw) + ly * LSTRIDE;
  SYNC sync;
  C v[E], prod[E];
  for (int op = 0; op < a.nop; ++op) {
    const C* base = (op == 0) ? a.in[0] : ((op == 1) ? a.in[1] : a.in[2]);
    const C* src = base + (long long)(valid ? line : 0) * a.in_stride;
    const int kin = valid ? a.kin : 0;
#pragma unroll
    for (int s = 0; s < E; ++s) v[s] = c2r_pre_g<T, H>(src, FI::in_index(t, s), kin, twM);
    FI::run(v, t, sm, 1, twH, sync);
    if (op == 0) {
#pragma unroll
      for (int s = 0; s < E; ++s) prod[s] = v[s];
    } else {
#pragma unroll
      for (int s = 0; s < E; ++s) { prod[s].x *= v[s].x; prod[s].y *= v[s].y; }
    }
  }
  // forward transform of the packed product: one exchange into stage-0 order
  sync();
#pragma unroll
  for (int s = 0; s < E; ++s) sm[FI::out_index(t, s)] = prod[s];
  sync();
#pragma unroll
  for (int s = 0; s < E; ++s) v[s] = sm[FF::in_index(t, s)];
  FF::run(v, t, sm, 1, twH, sync);
  sync();
#pragma unroll
  for (int s = 0; s < E; ++s) sm[FF::out_index(t, s)] = v[s];
  sync();
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

// ---------------------------------------------------------------------------
// TMA-pipelined fused z pass.  Persistent CTAs walk batches of LPB
// consecutive lines; the operands of the next batch are fetched by bulk
// asynchronous copies (cp.async.bulk, one per operand, completion counted on
// an mbarrier) into the other half of a double buffer while the current batch
// is transformed, so HBM traffic overlaps the FFT work.
// Shared memory: [2 mbarriers | stage[2][nop][LPB][kin] | exchange[LPB][H+1]]
// ---------------------------------------------------------------------------
template <typename T, int H>
__device__ __forceinline__ cplx<T> c2r_pre_s(const cplx<T>* src, int k, int kin, const cplx<T>* __restrict__ twM) {
  using C = cplx<T>;
  C A = (k < kin) ? src[k] : mkc<T>(T(0), T(0));
  C B = (H - k < kin) ? src[H - k] : mkc<T>(T(0), T(0));
  if (k == 0) { A.y = T(0); B.y = T(0); }
  B = cconj(B);
  const C Ev = cadd(A, B);
  const C Ov = cmulc(csub(A, B), twM[k]);
  return mkc<T>(Ev.x - Ov.y, Ev.y + Ov.x);
}

// Output slots of a line FFT held as k = t + TPL a(s): the r2c post-processing
// pairs Z[k] with Z[H - k], which then sits in lane (TPL - t) mod TPL of the
// same line group, slot a' = E - 1 - a (or (E - a) mod E in lane 0), so one
// warp shuffle per slot replaces a shared-memory round trip.
template <class F>
__host__ __device__ constexpr int zslot_a(int s) {
  return s / F::RL + (F::TPL > 0 ? (F::LEN / F::RL) / F::TPL : 0) * (s % F::RL);
}
template <class F>
__host__ __device__ constexpr bool zshfl_post_ok() {
  if (!(F::TPL <= 32 && 32 % F::TPL == 0 && (F::LEN / F::RL) % F::TPL == 0)) return false;
  bool seen[64] = {};
  if (F::E > 64) return false;
  for (int s = 0; s < F::E; ++s) {
    const int a = zslot_a<F>(s);
    if (a < 0 || a >= F::E || seen[a]) return false;
    seen[a] = true;
  }
  return true;
}
template <class F>
__host__ __device__ constexpr int zslot_of(int a) {
  for (int s = 0; s < F::E; ++s)
    if (zslot_a<F>(s) == a) return s;
  return 0;
}

// MODE 0: the fused convolution z pass above.
// MODE 1: the inverse transform of one operand only, its real line (M reals
//         as H packed pairs) stored to out[line * out_stride + m].
// MODE 2: the forward transform of one real line (H packed pairs, kin = H),
//         stored as kz < kout like MODE 0.
// CTAs per SM the FP32 r2c z pass (MODE 2) is compiled for: it exchanges in
// its staged input lines, so four fit by shared memory at 128 registers
// (0 elsewhere: no minimum, the compiler's register choice)
template <typename T, int MODE>
__host__ __device__ constexpr int zconv_tma_minb() {
  return sizeof(T) != 4 ? 0 : (MODE == 2 ? 4 : 0);
}
// the r2c mode exchanges in its staged input lines (kin = H) when the
// exchange stride of a line fits in one
template <int H, int MODE>
__host__ __device__ constexpr bool zconv_xchg_in_stage() {
  return MODE == 2 && zline_stride(H) <= H;
}
template <typename T, int H, int MAXR, int LPB, class SYNC, int MODE = 0, int KIN = 0>
__global__ void __launch_bounds__(LPB * LineFFT<T, H, true, MAXR>::TPL, zconv_tma_minb<T, MODE>())
k_zconv_tma(ZConvArgs<T> a, const cplx<T>* __restrict__ twH, const cplx<T>* __restrict__ twM) {
  constexpr int LAY = zlayout(H);
  using FI = LineFFT<T, H, true, MAXR, LAY, true>;
  using FF = LineFFT<T, H, false, MAXR, LAY, true>;
  using C = cplx<T>;
  constexpr int E = FI::E, TPL = FI::TPL;
  constexpr int LS = zline_stride(H);  // per-line exchange length
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
  const int nop = (MODE == 0) ? a.nop : 1;
  const int kin = KIN ? KIN : a.kin;  // line length (compiled in when KIN > 0)
  C* stage = reinterpret_cast<C*>(smem_raw + 128);
  const int per_op = LPB * kin;
  C* xchg = stage + 2 * nop * per_op;
  const int t = threadIdx.x % TPL, ly = threadIdx.x / TPL;
  C* const sm_x = xchg + ly * LS;
  const int nbatch = a.nlines / LPB;
  const unsigned bytes_op = (unsigned)(per_op * sizeof(C));
  const C* in0 = a.in[0];
  const C* in1 = a.in[1];
  const C* in2 = a.in[2];
  SYNC sync;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int b, int st) {
    mbar_arrive_expect_tx(&bars[st], (unsigned)nop * bytes_op);
    const long long off = (long long)b * per_op;
    tma_load_1d(stage + (st * nop + 0) * per_op, in0 + off, bytes_op, &bars[st]);
    if (nop > 1) tma_load_1d(stage + (st * nop + 1) * per_op, in1 + off, bytes_op, &bars[st]);
    if (nop > 2) tma_load_1d(stage + (st * nop + 2) * per_op, in2 + off, bytes_op, &bars[st]);
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < nbatch) issue(blockIdx.x, 0);
  int iter = 0;
  bool pending_other = false;
  for (int b = blockIdx.x; b < nbatch; b += gridDim.x, ++iter) {
    const int st = iter & 1;
    const int bn = b + gridDim.x;
    if (threadIdx.x == 0 && bn < nbatch) {
      fence_proxy_async_smem();
      issue(bn, st ^ 1);
    }
    pending_other = bn < nbatch;
    const bool ok = mbar_wait_bounded(&bars[st], (iter >> 1) & 1, a.err, 1);
    if (!__syncthreads_and(ok)) {
      // give the copy still in flight into the other buffer a bounded chance to land
      if (pending_other) mbar_wait_bounded(&bars[st ^ 1], ((iter + 1) >> 1) & 1, nullptr, 0);
      return;
    }
    C v[E], prod[E];
    // this line's exchange area: its staged input line in the r2c mode (read
    // into registers before the transform's first exchange), else its own
    C* const sm = zconv_xchg_in_stage<H, MODE>() ? stage + (st * nop) * per_op + ly * kin : sm_x;
    if constexpr (MODE == 2) {
      const C* src = stage + (st * nop) * per_op + ly * kin;
#pragma unroll
      for (int s = 0; s < E; ++s) v[s] = src[FF::in_index(t, s)];
    }
    const int nops = (MODE == 0) ? nop : (MODE == 1 ? 1 : 0);  // compile-time for the one-transform modes
    for (int op = 0; op < nops; ++op) {
      const C* src = stage + (st * nop + op) * per_op + ly * kin;
#pragma unroll
      for (int s = 0; s < E; ++s) v[s] = c2r_pre_s<T, H>(src, FI::in_index(t, s), kin, twM);
      FI::run(v, t, sm, 1, twH, sync);
      if (op == 0) {
#pragma unroll
        for (int s = 0; s < E; ++s) prod[s] = v[s];
      } else {
#pragma unroll
        for (int s = 0; s < E; ++s) { prod[s].x *= v[s].x; prod[s].y *= v[s].y; }
      }
    }
    if constexpr (MODE == 1) {
      C* dst = a.out + (long long)(b * LPB + ly) * a.out_stride;
#pragma unroll
      for (int s = 0; s < E; ++s) dst[FI::out_index(t, s)] = prod[s];
    } else {
      if constexpr (MODE == 0) {
        sync();
#pragma unroll
        for (int s = 0; s < E; ++s) sm[pidx<LAY>(FI::out_index(t, s))] = prod[s];
        sync();
#pragma unroll
        for (int s = 0; s < E; ++s) v[s] = sm[pidx<LAY>(FF::in_index(t, s))];
      }
      FF::run(v, t, sm, 1, twH, sync);
      C* dst = a.out + (long long)(b * LPB + ly) * a.out_stride;
      if constexpr (zshfl_post_ok<FF>()) {
        // Z[H - k] from the partner lane by shuffles (no exchange through shared memory)
        const int lane = threadIdx.x & 31;
        const int src = (lane & ~(TPL - 1)) + ((TPL - t) & (TPL - 1));
        // slots that can hold a kept k: the r2c mode keeps kz <= 2H/3 (the
        // Orszag N/2, checked at launch), the fused pass up to H
        constexpr int QK = (MODE == 2) ? (2 * H / 3 + 1 + TPL - 1) / TPL : E;
        constexpr int QMAX = QK < E ? QK : E;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
          const C give = (t == 0) ? v[zslot_of<FF>((E - q) % E)] : v[zslot_of<FF>(E - 1 - q)];
          C zc;
          zc.x = __shfl_sync(0xffffffffu, give.x, src);
          zc.y = -__shfl_sync(0xffffffffu, give.y, src);
          const int k = t + TPL * q;
          const C zk = v[zslot_of<FF>(q)];
          if (k < a.kout) {
            const C Ev = mkc<T>(T(0.5) * (zk.x + zc.x), T(0.5) * (zk.y + zc.y));
            const C Ov = mkc<T>(T(0.5) * (zk.y - zc.y), -T(0.5) * (zk.x - zc.x));
            dst[k] = cscale(cadd(Ev, cmul(twM[k], Ov)), a.out_scale);
          }
        }
        if (t == 0 && a.kout > H) {  // k = H (kept when kout = H + 1): Z[H] = Z[0]
          const C zk = v[zslot_of<FF>(0)];
          const C Ev = mkc<T>(zk.x, T(0));
          const C Ov = mkc<T>(zk.y, T(0));
          dst[H] = cscale(cadd(Ev, cmul(twM[H], Ov)), a.out_scale);
        }
        __syncthreads();  // stage[st] fully consumed before it is refilled
        continue;
      }
      sync();
#pragma unroll
      for (int s = 0; s < E; ++s) sm[pidx<LAY>(FF::out_index(t, s))] = v[s];
      sync();
      for (int k = t; k < a.kout; k += TPL) {
        const C zk = sm[pidx<LAY>(k % H)];
        const C zc = cconj(sm[pidx<LAY>((H - k) % H)]);
        const C Ev = mkc<T>(T(0.5) * (zk.x + zc.x), T(0.5) * (zk.y + zc.y));
        const C Ov = mkc<T>(T(0.5) * (zk.y - zc.y), -T(0.5) * (zk.x - zc.x));
        dst[k] = cscale(cadd(Ev, cmul(twM[k], Ov)), a.out_scale);
      }
    }
    __syncthreads();  // stage[st] fully consumed before it is refilled
  }
}

}  // namespace mf
