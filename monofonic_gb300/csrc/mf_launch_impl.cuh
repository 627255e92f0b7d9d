// Launch configuration and per-length dispatch of the FFT pass kernels.
// Each translation unit mf_fft_<part>_<prec>.cu defines MF_T and one MF_PART_*
// macro and includes this file, so the instantiations compile in parallel.
#pragma once

#include "mf_internal.h"
#include <type_traits>

// CTAs per SM the fused z pass is compiled for in FP32 (a build-time knob)
#ifndef MF_ZCONV_MINB_F32
#define MF_ZCONV_MINB_F32 2
#endif
// 1: persistent double-buffered (cp.async) strided passes (a build-time knob)
#ifndef MF_COL_PIPE
#define MF_COL_PIPE 1
#endif
// 1: TMA-pipelined fused z pass where the layout allows it (a build-time knob)
#ifndef MF_ZCONV_TMA
#define MF_ZCONV_TMA 1
#endif
// divisors of the lines per batch of the one-transform TMA z passes (build-time
// knobs): at N=512 quarter batches were 2 % faster for the c2r (MODE 1) and
// 8 % slower for the r2c (MODE 2) than half batches
#ifndef MF_ZONE_LPB_DIV
#define MF_ZONE_LPB_DIV 2
#endif
#ifndef MF_ZC2R_LPB_DIV
#define MF_ZC2R_LPB_DIV 4
#endif
// largest radix of the TMA z pass plan (8: fewer exchanges, more registers)
#ifndef MF_ZCONV_TMA_MAXR
#define MF_ZCONV_TMA_MAXR 8
#endif

#include "mf_kernels.cuh"
#include "mf_runtime.h"
#include "mf_sched.h"

namespace mf {

// columns per CTA of a strided pass: 128-byte rows (16 float2 / 8 double2),
// at most 1024 threads, at least 128 threads
template <typename T, int L>
constexpr int col_ncol() {
  constexpr int tpl = LineFFT<T, L, false>::TPL;
  int nc = (sizeof(T) == 4) ? 16 : 8;
  while (nc * tpl > 1024) nc /= 2;
  while (nc * tpl < 128 && nc < 64) nc *= 2;
  return nc;
}

// lines per CTA of a z pass, bounded by ~100 KB of shared memory per CTA
template <typename T, int H, int SMEM_ELEMS_PER_LINE>
constexpr int z_lpb() {
  constexpr int tpl = LineFFT<T, H, false>::TPL;
  int l = 256 / tpl;
  if (l < 1) l = 1;
  while (l > 1 && (size_t)l * SMEM_ELEMS_PER_LINE * sizeof(cplx<T>) > 100 * 1024) l /= 2;
  return l;
}

template <typename K>
inline cudaError_t set_smem(K kern, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

// row bytes of a tile of the pipelined strided pass (a build-time knob)
#ifndef MF_PIPE_ROW_BYTES
#define MF_PIPE_ROW_BYTES 64
#endif
// columns per CTA of the pipelined strided pass (two tile buffers): rows of
// MF_PIPE_ROW_BYTES while both buffers fit in 220 KB, at least 128 threads
template <typename T, int L>
constexpr int pipe_ncol() {
  constexpr int tpl = LineFFT<T, L, false, MF_COL_MAXR>::TPL;
  int nc = MF_PIPE_ROW_BYTES / (int)(2 * sizeof(T));
  while (nc > 1 && (nc * tpl > 1024 || 2 * L * nc * (int)(2 * sizeof(T)) > 220 * 1024)) nc /= 2;
  while (nc * tpl < 128 && nc < 32) nc *= 2;
  return nc;
}

// 1: the pipelined strided passes with one column per warp where eligible
// (k_colfft_wpc; a build-time knob)
#ifndef MF_COL_WPC
#define MF_COL_WPC 0
#endif

template <typename T, int L, bool INV, class OP>
cudaError_t launch_col(OP op, int nslab, int ncols, int nz, const cplx<T>* tw, cudaStream_t s, int kind) {
  if constexpr (OP::kPipe && MF_COL_PIPE && MF_COL_WPC && wpc_ok<T, L, INV, OP>()) {
    constexpr int NC = pipe_ncol<T, L>();
    constexpr int TPL = LineFFT<T, L, INV, MF_COL_MAXR>::TPL;
    const size_t smem = (size_t)2 * NC * wpc_lsc<T, L, INV>() * sizeof(cplx<T>);
    auto kern = k_colfft_wpc<T, L, INV, NC, OP>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NC * TPL, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const int ntc = (ncols + NC - 1) / NC;
    const int total = ntc * nslab * nz;
    int grid = nsm * per_sm;
    if (grid > total) grid = total;
    kern<<<grid, NC * TPL, smem, s>>>(op, tw, ncols, ntc, nslab, nz);
    return cudaGetLastError();
  } else if constexpr (OP::kPipe && MF_COL_PIPE) {
    constexpr int NC = pipe_ncol<T, L>();
    constexpr int TPL = LineFFT<T, L, INV, MF_COL_MAXR>::TPL;
    const size_t smem = (size_t)2 * L * NC * sizeof(cplx<T>);
    auto kern = k_colfft_pipe<T, L, INV, NC, OP>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NC * TPL, smem);
    if (e != cudaSuccess) return e;
    const PassSched sc = sched_get(kind, L, (int)sizeof(T));
    if (sc.occ > 0 && sc.occ < per_sm) per_sm = sc.occ;
    if (per_sm < 1) per_sm = 1;
    const int ntc = (ncols + NC - 1) / NC;
    const int total = ntc * nslab * nz;
    int grid = nsm * per_sm;
    if (grid > total) grid = total;
    dim3 block(NC, TPL);
    kern<<<grid, block, smem, s>>>(op, tw, ncols, ntc, nslab, nz);
    return cudaGetLastError();
  } else {
    constexpr int NC = col_ncol<T, L>();
    constexpr int TPL = LineFFT<T, L, INV>::TPL;
    const size_t smem = (size_t)L * NC * sizeof(cplx<T>);
    auto kern = k_colfft<T, L, INV, NC, OP>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    dim3 block(NC, TPL), grid((ncols + NC - 1) / NC, nslab, nz);
    kern<<<grid, block, smem, s>>>(op, tw, ncols);
    return cudaGetLastError();
  }
}

// N-grid lengths, and the convolution pass lengths that have a compile-time
// geometry: Orszag M = 3N/2 and aliased M = N for an N-grid length N
__host__ __device__ constexpr bool ngrid_len(int L) {
  return L == 16 || L == 32 || L == 64 || L == 96 || L == 128 || L == 192 || L == 256 || L == 384 || L == 512;
}
__host__ __device__ constexpr bool orszag_len(int L) { return L % 3 == 0 && ngrid_len(2 * L / 3); }

// a convolution pass of length L (the padded axis, M = L) launched with its
// geometry as compile-time constants; a geometry that is neither the Orszag
// nor the aliased form of a compiled length is refused
template <typename T, int L, class LAUNCH, class OP>
cudaError_t with_conv_geom(const OP& op, LAUNCH&& go) {
  if (op.g.orszag) {
    if constexpr (orszag_len(L)) {
      using G = CGeom<L, true>;
      if (!geom_matches<G>(op.g)) return cudaErrorInvalidValue;
      return go(op.template with_geom<G>());
    }
    return cudaErrorInvalidValue;
  }
  if constexpr (ngrid_len(L)) {
    using G = CGeom<L, false>;
    if (!geom_matches<G>(op.g)) return cudaErrorInvalidValue;
    return go(op.template with_geom<G>());
  }
  return cudaErrorInvalidValue;
}

// a plain strided pass of length L launched with compile-time strides when
// they are those of an x or y pass over an L-grid, else with its own
template <typename T, int L, class LAUNCH>
cudaError_t with_plain_axis(const PlainStridedOp<T>& op, LAUNCH&& go) {
  const long long kz = L / 2 + 1;
  if (op.e_str == (long long)L * kz && op.slab_str == kz) return go(op.template with_axis<L, 0>());
  if (op.e_str == kz && op.slab_str == (long long)L * kz) return go(op.template with_axis<L, 1>());
  return go(op);
}

template <typename T, int H, class OP>
cudaError_t launch_zr2c(OP op, int nlines, int kout, const cplx<T>* twH, const cplx<T>* twM, cudaStream_t s) {
  constexpr int LPB = z_lpb<T, H, H + 1>();
  constexpr int TPL = LineFFT<T, H, false>::TPL;
  const size_t smem = (size_t)LPB * (H + 1) * sizeof(cplx<T>);
  auto kern = k_zr2c<T, H, TPL * LPB, OP>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  dim3 block(TPL, LPB), grid((nlines + LPB - 1) / LPB);
  kern<<<grid, block, smem, s>>>(op, twH, twM, nlines, kout);
  return cudaGetLastError();
}

template <typename T, int H, class OP>
cudaError_t launch_zc2r(OP op, int nlines, int kin, const cplx<T>* twH, const cplx<T>* twM, cudaStream_t s) {
  constexpr int LPB = z_lpb<T, H, H + 1>();
  constexpr int TPL = LineFFT<T, H, true>::TPL;
  const size_t smem = (size_t)LPB * (H + 1) * sizeof(cplx<T>);
  auto kern = k_zc2r<T, H, TPL * LPB, OP>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  dim3 block(TPL, LPB), grid((nlines + LPB - 1) / LPB);
  kern<<<grid, block, smem, s>>>(op, twH, twM, nlines, kin);
  return cudaGetLastError();
}

// lines per batch of the TMA z pass: a power of two >= 2 (so a batch of
// FP32 lines of odd length is a multiple of 16 bytes), ~256 FP32 / ~128 FP64
// threads per CTA
template <typename T, int TPL>
constexpr int tma_lines_per_batch() {
  const int target = ((sizeof(T) == 4) ? 256 : 128) / TPL;
  int l = 2;
  while (l * 2 <= target) l *= 2;
  return l;
}

// fused z pass: the TMA-pipelined persistent kernel when every batch of LPB
// lines is one 16-byte aligned contiguous block per operand, otherwise the
// direct-load kernel.  Radix-4 plan (fewer registers per thread); warp
// barriers when a line's threads fit in one warp.
// MODE 1 / 2: the shared-source inverse transform of one operand into a real
// padded field / forward transform of one real padded field (fallbacks: the
// direct-load plain z kernels)
template <typename T, int H, int MODE = 0>
cudaError_t launch_zconv(const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM, cudaStream_t s) {
  const PassSched sc = sched_get(KK_CONV_Z, 2 * H, (int)sizeof(T));
  if (sc.variant == 0 || MODE != 0) {
    // TMA path: radix-8-first plan with the padded (conflict-free) exchange layout
    constexpr int MAXR = MF_ZCONV_TMA_MAXR;
    constexpr int TPL = LineFFT<T, H, true, MAXR>::TPL;
    constexpr bool WARP = (TPL <= 32) && (32 % TPL == 0);
    using SYNC = typename std::conditional<WARP, SyncWarp, SyncBlock>::type;
    // lines per batch; the one-transform modes may use a fraction of it (a
    // build-time knob: more, smaller CTAs per SM)
    constexpr int LPB0 = tma_lines_per_batch<T, TPL>();
    constexpr int DIV = (MODE == 1) ? MF_ZC2R_LPB_DIV : MF_ZONE_LPB_DIV;
    constexpr int LPBT = (MODE != 0 && LPB0 >= 2 * DIV) ? LPB0 / DIV : LPB0;
    // (the r2c mode's lines hold H pairs; its exchanges run in them when they fit)
    const bool tma_ok = MF_ZCONV_TMA && (MODE != 2 || (a.kin == H && a.kout <= 2 * H / 3 + 1)) &&
                        (a.nlines % LPBT == 0) && (a.in_stride == a.kin) &&
                        (((size_t)LPBT * a.kin * sizeof(cplx<T>)) % 16 == 0) &&
                        ((uintptr_t)a.in[0] % 16 == 0) && (a.nop < 2 || (uintptr_t)a.in[1] % 16 == 0) &&
                        (a.nop < 3 || (uintptr_t)a.in[2] % 16 == 0);
    if (tma_ok) {
      // the c2r of one Orszag operand with its line length (kz <= N/2, 2H/3 + 1)
      // compiled in: 0.561 -> 0.520 ms per launch at N=512 (the r2c with its H
      // pairs compiled in measured no faster)
      constexpr int KIN_CT = (MODE == 1 && H % 3 == 0) ? 2 * H / 3 + 1 : 0;
      auto kern = (KIN_CT != 0 && a.kin == KIN_CT) ? k_zconv_tma<T, H, MAXR, LPBT, SYNC, MODE, KIN_CT>
                                                   : k_zconv_tma<T, H, MAXR, LPBT, SYNC, MODE, 0>;
      const size_t smem =
          128 + ((size_t)2 * a.nop * LPBT * a.kin + (zconv_xchg_in_stage<H, MODE>() ? 0 : (size_t)LPBT * zline_stride(H))) *
                    sizeof(cplx<T>);
      cudaError_t e = set_smem(kern, smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, nsm = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, LPBT * TPL, smem);
      if (e != cudaSuccess) return e;
      // the autotuned CTAs per SM belong to the fused convolution pass (MODE 0)
      if (MODE == 0 && sc.occ > 0 && sc.occ < per_sm) per_sm = sc.occ;
      if (per_sm < 1) per_sm = 1;
      const int nbatch = a.nlines / LPBT;
      int grid = nsm * per_sm;
      if (grid > nbatch) grid = nbatch;
      kern<<<grid, LPBT * TPL, smem, s>>>(a, twH, twM);
      return cudaGetLastError();
    }
  }
  if constexpr (MODE == 1) {
    return launch_zc2r<T, H>(PadC2RZOp<T>{a.in[0], a.in_stride, a.out, (int)a.out_stride}, a.nlines, a.kin, twH,
                             twM, s);
  }
  if constexpr (MODE == 2) {
    return launch_zr2c<T, H>(PadR2CZOp<T>{a.in[0], (int)a.in_stride, a.out, a.out_stride}, a.nlines, a.kout, twH,
                             twM, s);
  }
  // direct-load fallback: radix-4 plan, unpadded
  constexpr int MAXR = 4;
  constexpr int TPL = LineFFT<T, H, true, MAXR>::TPL;
  constexpr bool WARP = (TPL <= 32) && (32 % TPL == 0);
  using SYNC = typename std::conditional<WARP, SyncWarp, SyncBlock>::type;
  constexpr int NT = (TPL >= 256) ? TPL : (256 / TPL) * TPL;
  constexpr int LPB = NT / TPL;
  const size_t smem = (size_t)LPB * (H + 1) * sizeof(cplx<T>);
  constexpr int MINB = (sizeof(T) == 4) ? MF_ZCONV_MINB_F32 : 1;
  auto kern = k_zconv<T, H, MAXR, NT, MINB, SYNC>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<(a.nlines + LPB - 1) / LPB, NT, smem, s>>>(a, twH, twM);
  return cudaGetLastError();
}

// compiled lengths: N-grid passes (L = N, H = N/2) and convolution passes
// (L = M for Orszag 3/2, M = N for the aliased convolver)
#define MF_LEN_N(X) X(16) X(32) X(64) X(96) X(128) X(192) X(256) X(384) X(512)
#define MF_LEN_NH(X) X(8) X(16) X(32) X(48) X(64) X(96) X(128) X(192) X(256)
#define MF_LEN_CONV(X) \
  X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(144) X(192) X(256) X(288) X(384) X(512) X(576) X(768)
#define MF_LEN_CONVH(X) \
  X(8) X(12) X(16) X(24) X(32) X(48) X(64) X(72) X(96) X(128) X(144) X(192) X(256) X(288) X(384)

#if defined(MF_PART_PLAIN)
template <typename T>
cudaError_t Launch<T>::colfft_plain(int L, bool inv, PlainStridedOp<T> op, int nslab, int ncols,
                                    const cplx<T>* tw, cudaStream_t s) {
#define CASE(LL)                                                                     \
  case LL:                                                                           \
    return with_plain_axis<T, LL>(op, [&](auto o) {                                  \
      return inv ? launch_col<T, LL, true>(o, nslab, ncols, 1, tw, s, KK_FFT_COL)      \
                 : launch_col<T, LL, false>(o, nslab, ncols, 1, tw, s, KK_FFT_COL);    \
    });
  switch (L) { MF_LEN_N(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::z_r2c_plain(int H, PlainZOp<T> op, int nlines, int kout, const cplx<T>* twH,
                                   const cplx<T>* twM, cudaStream_t s) {
#define CASE(HH) case HH: return launch_zr2c<T, HH>(op, nlines, kout, twH, twM, s);
  switch (H) { MF_LEN_NH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::z_c2r_plain(int H, PlainZOp<T> op, int nlines, int kin, const cplx<T>* twH,
                                   const cplx<T>* twM, cudaStream_t s) {
#define CASE(HH) case HH: return launch_zc2r<T, HH>(op, nlines, kin, twH, twM, s);
  switch (H) { MF_LEN_NH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::assemble_xinv(int L, AssembleXInvOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                     cudaStream_t s) {
#define CASE(LL) case LL: return launch_col<T, LL, true>(op, nslab, ncols, 1, tw, s, KK_FFT_COL);
  switch (L) { MF_LEN_N(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T, int L>
cudaError_t launch_col3(Assemble3XInvOp<T> op, int nslab, int ncols, const cplx<T>* tw, cudaStream_t s) {
  if constexpr (LineFFT<T, L, true>::E > 8) {
    return cudaErrorInvalidValue;  // three register sets of E > 8 elements: per-component passes instead
  } else {
    // at most 512 threads, so that the three register sets fit without spilling
    constexpr int TPL = LineFFT<T, L, true>::TPL;
    constexpr int NC0 = col_ncol<T, L>();
    constexpr int NC = (NC0 * TPL > 512) ? ((512 / TPL) > 0 ? 512 / TPL : 1) : NC0;
    dim3 block(NC, TPL), grid((ncols + NC - 1) / NC, nslab, 1);
    if (op.n == L && op.Kz == L / 2 + 1) {
      // the grid as compile-time constants, components staged through shared
      // memory (two CTAs per SM where three tiles fit twice)
      const size_t smem = (size_t)3 * L * NC * sizeof(cplx<T>);
      constexpr int MINB = (2 * 3 * L * NC * (int)sizeof(cplx<T>) <= 200 * 1024 && NC * TPL <= 512) ? 2 : 1;
      auto kern = k_colfft3s<T, L, true, NC, Assemble3XInvOp<T, L>, MINB>;
      cudaError_t e = set_smem(kern, smem);
      if (e != cudaSuccess) return e;
      kern<<<grid, block, smem, s>>>(op.template with_n<L>(), tw, ncols);
      return cudaGetLastError();
    }
    const size_t smem = (size_t)L * NC * sizeof(cplx<T>);
    auto kern = k_colfft3<T, L, true, NC, Assemble3XInvOp<T>>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, block, smem, s>>>(op, tw, ncols);
    return cudaGetLastError();
  }
}
template <typename T>
bool Launch<T>::assemble3_supported(int L) {
#define CASE(LL) case LL: return LineFFT<T, LL, true>::E <= 8;
  switch (L) { MF_LEN_N(CASE) default: return false; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::assemble3_xinv(int L, Assemble3XInvOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                      cudaStream_t s) {
#define CASE(LL) case LL: return launch_col3<T, LL>(op, nslab, ncols, tw, s);
  switch (L) { MF_LEN_N(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T, int H>
cudaError_t launch_zc2r3_lattice(const Lattice3Args& a, bool p64, const cplx<T>* twH, const cplx<T>* twM,
                                 cudaStream_t s) {
  // lines per batch: at most 256 threads, two batch buffers within ~100 KB so
  // that two CTAs share an SM
  constexpr int TPL = LineFFT<T, H, true>::TPL;
  constexpr int LPB = [] {
    int l = 256 / TPL;
    if (l < 1) l = 1;
    while (l > 1 && 2 * (size_t)l * 3 * (H + 1) * sizeof(cplx<T>) > 100 * 1024) l /= 2;
    return l;
  }();
  const size_t smem = (size_t)2 * LPB * 3 * (H + 1) * sizeof(cplx<T>);
  if (a.nlines % LPB) return cudaErrorInvalidValue;  // whole batches (n^2 lines, n even)
  const int nb = a.nlines / LPB;
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPL * LPB, smem);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(nb, std::max(1, per_sm) * nsm));
    kern<<<grid, dim3(TPL, LPB), smem, s>>>(a, twH, twM);
    return cudaGetLastError();
  };
  return p64 ? go(k_zc2r3_lattice<T, H, LPB, double>) : go(k_zc2r3_lattice<T, H, LPB, float>);
}
template <typename T>
cudaError_t Launch<T>::z_c2r3_lattice(int H, const Lattice3Args& a, bool p64, const cplx<T>* twH,
                                      const cplx<T>* twM, cudaStream_t s) {
#define CASE(HH) case HH: return launch_zc2r3_lattice<T, HH>(a, p64, twH, twM, s);
  switch (H) { MF_LEN_NH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template cudaError_t Launch<MF_T>::z_c2r3_lattice(int, const Lattice3Args&, bool, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
template bool Launch<MF_T>::assemble3_supported(int);
template cudaError_t Launch<MF_T>::assemble3_xinv(int, Assemble3XInvOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::colfft_plain(int, bool, PlainStridedOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::assemble_xinv(int, AssembleXInvOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::z_r2c_plain(int, PlainZOp<MF_T>, int, int, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::z_c2r_plain(int, PlainZOp<MF_T>, int, int, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
#endif

#if defined(MF_PART_CONVX)
template <typename T>
cudaError_t Launch<T>::conv_xinv(int L, ConvXInvOp<T> op, int nslab, int ncols, int nops,
                                 const cplx<T>* tw, cudaStream_t s) {
#define CASE(LL)                                                                                        \
  case LL:                                                                                             \
    return with_conv_geom<T, LL>(op, [&](auto o) { return launch_col<T, LL, true>(o, nslab, ncols, nops, tw, s, KK_CONV_XINV); });
  switch (L) { MF_LEN_CONV(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::conv_xfwd(int L, ConvXFwdOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                 cudaStream_t s) {
#define CASE(LL)                                                                                        \
  case LL:                                                                                             \
    return with_conv_geom<T, LL>(op, [&](auto o) { return launch_col<T, LL, false>(o, nslab, ncols, 1, tw, s, KK_CONV_XFWD); });
  switch (L) { MF_LEN_CONV(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T, int L, class OP>
cudaError_t launch_xtrunc(OP op, int nslab, int ncols, const cplx<T>* tw, cudaStream_t s) {
  constexpr int NC = pipe_ncol<T, L>();
  constexpr int TPL = LineFFT<T, L, false, MF_COL_MAXR>::TPL;
  const size_t smem = (size_t)2 * L * NC * sizeof(cplx<T>);
  auto kern = k_colfft_trunc<T, L, NC, OP>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0, nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NC * TPL, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int ntc = (ncols + NC - 1) / NC;
  const int total = ntc * nslab;
  int grid = nsm * per_sm;
  if (grid > total) grid = total;
  kern<<<grid, dim3(NC, TPL), smem, s>>>(op, tw, ncols, ntc, nslab);
  return cudaGetLastError();
}
template <typename T>
cudaError_t Launch<T>::conv_xtrunc(int L, ConvXTruncOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                   cudaStream_t s) {
#define CASE(LL)                                                                                        \
  case LL:                                                                                             \
    return with_conv_geom<T, LL>(op, [&](auto o) { return launch_xtrunc<T, LL>(o, nslab, ncols, tw, s); });
  switch (L) { MF_LEN_CONV(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template cudaError_t Launch<MF_T>::conv_xinv(int, ConvXInvOp<MF_T>, int, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::conv_xfwd(int, ConvXFwdOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::conv_xtrunc(int, ConvXTruncOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
#endif

#if defined(MF_PART_CONVY)
template <typename T>
cudaError_t Launch<T>::conv_yinv(int L, ConvYInvOp<T> op, int nslab, int ncols, int nops,
                                 const cplx<T>* tw, cudaStream_t s) {
#define CASE(LL)                                                                                        \
  case LL:                                                                                             \
    return with_conv_geom<T, LL>(op, [&](auto o) { return launch_col<T, LL, true>(o, nslab, ncols, nops, tw, s, KK_CONV_YINV); });
  switch (L) { MF_LEN_CONV(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::conv_yfwd(int L, ConvYFwdOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                 cudaStream_t s) {
#define CASE(LL)                                                                                        \
  case LL:                                                                                             \
    return with_conv_geom<T, LL>(op, [&](auto o) { return launch_col<T, LL, false>(o, nslab, ncols, 1, tw, s, KK_CONV_YFWD); });
  switch (L) { MF_LEN_CONV(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template cudaError_t Launch<MF_T>::conv_yinv(int, ConvYInvOp<MF_T>, int, int, int, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::conv_yfwd(int, ConvYFwdOp<MF_T>, int, int, const cplx<MF_T>*, cudaStream_t);
#endif

#if defined(MF_PART_ZCONV)
template <typename T>
cudaError_t Launch<T>::z_conv(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                              cudaStream_t s) {
#define CASE(HH) case HH: return launch_zconv<T, HH>(a, twH, twM, s);
  switch (H) { MF_LEN_CONVH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template cudaError_t Launch<MF_T>::z_conv(int, const ZConvArgs<MF_T>&, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
template <typename T>
cudaError_t Launch<T>::z_c2r_tma(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                                 cudaStream_t s) {
#define CASE(HH) case HH: return launch_zconv<T, HH, 1>(a, twH, twM, s);
  switch (H) { MF_LEN_CONVH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template <typename T>
cudaError_t Launch<T>::z_r2c_tma(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                                 cudaStream_t s) {
#define CASE(HH) case HH: return launch_zconv<T, HH, 2>(a, twH, twM, s);
  switch (H) { MF_LEN_CONVH(CASE) default: return cudaErrorInvalidValue; }
#undef CASE
}
template cudaError_t Launch<MF_T>::z_c2r_tma(int, const ZConvArgs<MF_T>&, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
template cudaError_t Launch<MF_T>::z_r2c_tma(int, const ZConvArgs<MF_T>&, const cplx<MF_T>*, const cplx<MF_T>*, cudaStream_t);
#endif

}  // namespace mf
