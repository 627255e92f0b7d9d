// Internal host-side interfaces shared by the translation units of libmfgpu.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "mf_fft.cuh"
#include "mf_ops.cuh"

namespace mf {

// status codes of the C ABI (mirrors include/monofonic_gb300.h)
enum Status : int {
  ST_OK = 0,
  ST_ERR_ARG = 1,
  ST_ERR_SHAPE = 2,
  ST_ERR_OOM = 3,
  ST_ERR_CUDA = 4,
  ST_ERR_TIMEOUT = 5,
  ST_ERR_CANCELLED = 6,
  ST_ERR_STATE = 7,
};

// FFT lengths for which kernels are compiled
bool length_supported(int L);
// grid sizes N the pipeline supports (N, 3N/2, N/2, 3N/4 all compiled)
bool grid_size_supported(int n);

// per-context twiddle tables w_L^j = exp(-2 pi i j / L), j in [0, L)
class TwiddleCache {
 public:
  ~TwiddleCache();
  const double2* get64(int L, cudaStream_t s);
  const float2* get32(int L, cudaStream_t s);
  template <typename T> const cplx<T>* get(int L, cudaStream_t s);
  void release();

 private:
  std::map<int, double2*> t64_;
  std::map<int, float2*> t32_;
  std::mutex mu_;
};

// precision-templated launchers (defined in mf_fft_<prec>.cu)
template <typename T>
struct Launch {
  // strided pass kinds
  static cudaError_t colfft_plain(int L, bool inv, PlainStridedOp<T> op, int nslab, int ncols,
                                  const cplx<T>* tw, cudaStream_t s);
  static cudaError_t assemble_xinv(int L, AssembleXInvOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                   cudaStream_t s);
  // all three components in one launch (lengths whose plan keeps E <= 8)
  static bool assemble3_supported(int L);
  static cudaError_t assemble3_xinv(int L, Assemble3XInvOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                    cudaStream_t s);
  // z c2r of the three components with the lattice readout fused (H = n/2);
  // p64: double positions / velocities (and fields mode)
  static cudaError_t z_c2r3_lattice(int H, const Lattice3Args& a, bool p64, const cplx<T>* twH, const cplx<T>* twM,
                                    cudaStream_t s);
  static cudaError_t conv_xinv(int L, ConvXInvOp<T> op, int nslab, int ncols, int nops,
                               const cplx<T>* tw, cudaStream_t s);
  static cudaError_t conv_yinv(int L, ConvYInvOp<T> op, int nslab, int ncols, int nops,
                               const cplx<T>* tw, cudaStream_t s);
  static cudaError_t conv_yfwd(int L, ConvYFwdOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                               cudaStream_t s);
  static cudaError_t conv_xfwd(int L, ConvXFwdOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                               cudaStream_t s);
  // convolve3's truncation of a pair product: x r2c pass, unpad, pad, x c2r pass
  static cudaError_t conv_xtrunc(int L, ConvXTruncOp<T> op, int nslab, int ncols, const cplx<T>* tw,
                                 cudaStream_t s);
  // z passes
  static cudaError_t z_r2c_plain(int H, PlainZOp<T> op, int nlines, int kout, const cplx<T>* twH,
                                 const cplx<T>* twM, cudaStream_t s);
  static cudaError_t z_c2r_plain(int H, PlainZOp<T> op, int nlines, int kin, const cplx<T>* twH,
                                 const cplx<T>* twM, cudaStream_t s);
  static cudaError_t z_conv(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                            cudaStream_t s);
  // z passes of the shared-source convolutions (padded lengths):
  // c2r of one operand line set into a real padded field (a.nop = 1, a.out = real field)
  static cudaError_t z_c2r_tma(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                               cudaStream_t s);
  // r2c of one real padded field, kz < a.kout kept (a.nop = 1, a.in[0] = real field)
  static cudaError_t z_r2c_tma(int H, const ZConvArgs<T>& a, const cplx<T>* twH, const cplx<T>* twM,
                               cudaStream_t s);
};

}  // namespace mf
