// Host-side objects behind the C ABI handles.
#pragma once

#include <cuda_runtime.h>
#include <string>
#include <utility>
#include <vector>

#include "../../include/monofonic_gb300.h"
#include "mf_internal.h"

namespace mf {
// kernel kinds for launch counting and in-stream event profiling
enum KernelKind : int {
  KK_CONV_XINV = 0,
  KK_CONV_YINV = 1,
  KK_CONV_Z = 2,
  KK_CONV_YFWD = 3,
  KK_CONV_XFWD = 4,
  KK_FFT_Z = 5,
  KK_FFT_COL = 6,
  KK_POINTWISE = 7,
  KK_COUNT = 8
};
}  // namespace mf

struct mf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  mf::TwiddleCache tw;
  std::string err;
  int children = 0;  // live grids, convolvers and pipelines on this context
  int* d_err = nullptr;  // device error flag set by bounded waits in kernels
  bool capturing = false;  // work is being recorded into a CUDA graph (no profiling events)
  // launch accounting
  long long launches[mf::KK_COUNT] = {};
  bool profile = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_events;
  std::vector<cudaEvent_t> event_pool;
};

namespace mf {
// RAII bracket of one kernel launch: counts it and, when profiling is on,
// records an event pair around it on the context's stream
class LaunchScope {
 public:
  LaunchScope(mf_ctx* c, int kind);
  ~LaunchScope();

 private:
  mf_ctx* c_;
  int kind_;
  cudaEvent_t e1_ = nullptr;
};
}  // namespace mf

struct mf_grid {
  mf_ctx* ctx = nullptr;
  int n = 0;
  double L = 0;
  int prec = MF_PREC_F64;
  int space = MF_SPACE_R;
  void* d = nullptr;
  size_t bytes = 0;
};

struct mf_conv {
  mf_ctx* ctx = nullptr;
  int n = 0;
  double L = 0;
  int prec = MF_PREC_F64;
  int kind = MF_CONV_ORSZAG;
  void* work = nullptr;   // nbuf * M*M*(n/2+1) complex
  size_t work_bytes = 0;
  int nbuf = 0;
  mf_grid* fbuf = nullptr;  // N-grid intermediate of convolve3
};

namespace mf {

int set_err(mf_ctx* c, int code, const std::string& msg);
// synchronises the context's stream and turns a raised device error flag
// (a bounded wait that ran out) into MF_ERR_TIMEOUT; clears the flag
int check_device_error(mf_ctx* c);
int cuda_err(mf_ctx* c, cudaError_t e, const char* where);

inline size_t grid_reals(int n) { return (size_t)(n + 2) * n * n; }
inline size_t prec_size(int prec) { return prec == MF_PREC_F32 ? 4 : 8; }

// 3D transforms on an n-grid in the padded in-place layout (unitary)
template <typename T> cudaError_t fft3d_r2c(mf_ctx* c, T* data, int n);
template <typename T> cudaError_t fft3d_c2r(mf_ctx* c, T* data, int n);

// convolution on k-space N-grids
template <typename T>
cudaError_t conv_run(mf_conv* cv, const Operand<T>* ops, int nop, cplx<T>* target, int out_op, T x,
                     int post_invlap);

// pointwise kernels (mf_pointwise.cu)
template <typename T> cudaError_t pw_scale(T* d, size_t nreal, T x, cudaStream_t s);
template <typename T> cudaError_t pw_zero_dc(T* d, cudaStream_t s);
template <typename T> cudaError_t pw_invlap(cplx<T>* d, int n, double kfac, cudaStream_t s);
template <typename T> cudaError_t pw_shift(cplx<T>* d, int n, double kfac, double dx, const double sh[3], cudaStream_t s);
template <typename T> cudaError_t pw_fill_from_f64(T* d, const double* src, int n, cudaStream_t s);
// LPT source products over the shared padded real fields (mf_sources.cu):
// fields[0..16] (Hessians of phi, of phi(2), convolve3 pair products), outs
// the product sums of the set: SRC_PHI2 1, SRC_PAIRS 5, SRC_PHI3_A3 4,
// SRC_PHI2_PAIRS 6 (the phi(2) source and the five pairs in one pass)
enum { SRC_PHI2 = 0, SRC_PAIRS = 1, SRC_PHI3_A3 = 2, SRC_PHI2_PAIRS = 3 };
constexpr int kSrcFields = 17, kSrcOutputs = 6;
template <typename T>
cudaError_t pw_sources(int set, const T* const* fields, T* const* outs, size_t n, cudaStream_t s);

// project RNG plugin on the device (bit-identical to mf_white_noise_host);
// seed from *seed_dev when it is not null
template <typename T>
cudaError_t pw_white_noise(T* d, int n, unsigned long long seed, const unsigned long long* seed_dev, cudaStream_t s);
template <typename T>
cudaError_t pw_power_spectrum(const cplx<T>* d, int n, double kfac, int nbins, double* acc /*4*nbins*/, cudaStream_t s);

}  // namespace mf
