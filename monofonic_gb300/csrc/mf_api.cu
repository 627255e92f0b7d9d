// C ABI of libmfgpu: context, Grid_FFT and convolver handles.
#include <sys/mman.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "mf_runtime.h"

#define MF_VERSION_STR "monofonic_gb300 0.1 (sm_103a)"

namespace mf {

int set_err(mf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_err(mf_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return ST_OK;
  const int code = (e == cudaErrorMemoryAllocation) ? ST_ERR_OOM : ST_ERR_CUDA;
  return set_err(c, code, std::string(where) + ": " + cudaGetErrorString(e));
}

int check_device_error(mf_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "stream synchronize");
  int flag = 0;
  e = cudaMemcpy(&flag, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_err(c, e, "device error flag");
  if (flag) {
    cudaMemset(c->d_err, 0, sizeof(int));
    return set_err(c, ST_ERR_TIMEOUT, "a bounded device wait ran out (asynchronous copy did not complete)");
  }
  return ST_OK;
}

LaunchScope::LaunchScope(mf_ctx* c, int kind) : c_(c), kind_(kind) {
  ++c_->launches[kind];
  if (c_->profile && !c_->capturing) {
    cudaEvent_t e0 = nullptr;
    if (c_->event_pool.size() >= 2) {
      e0 = c_->event_pool.back(); c_->event_pool.pop_back();
      e1_ = c_->event_pool.back(); c_->event_pool.pop_back();
    } else {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1_);
    }
    cudaEventRecord(e0, c_->stream);
    c_->prof_events.push_back({kind_, {e0, e1_}});
  }
}

LaunchScope::~LaunchScope() {
  if (e1_) cudaEventRecord(e1_, c_->stream);
}

bool length_supported(int L) {
  switch (L) {
    case 8: case 12: case 16: case 24: case 32: case 48: case 64: case 72: case 96: case 128: case 144:
    case 192: case 256: case 288: case 384: case 512: case 576: case 768:
      return true;
    default:
      return false;
  }
}

bool grid_size_supported(int n) {
  switch (n) {
    case 16: case 32: case 64: case 96: case 128: case 192: case 256: case 384: case 512:
      return true;
    default:
      return false;
  }
}

// ---------------------------------------------------------------------------
// twiddles exp(-2 pi i j / L), generated on the host in extended precision
// ---------------------------------------------------------------------------
static void twiddle_host(int L, std::vector<double>& re, std::vector<double>& im) {
  re.resize(L);
  im.resize(L);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int j = 0; j < L; ++j) {
    // reduce to the first octant for accuracy
    const long double a = 2.0L * pi * (long double)j / (long double)L;
    re[j] = (double)cosl(a);
    im[j] = (double)(-sinl(a));
  }
  // exact values on the axes
  for (int j = 0; j < L; ++j) {
    if ((4 * j) % L == 0) {
      const int q = (4 * j) / L;
      const double c[4] = {1, 0, -1, 0}, s[4] = {0, -1, 0, 1};
      re[j] = c[q];
      im[j] = s[q];
    }
  }
}

TwiddleCache::~TwiddleCache() { release(); }

void TwiddleCache::release() {
  std::lock_guard<std::mutex> lk(mu_);
  for (auto& kv : t64_) cudaFree(kv.second);
  for (auto& kv : t32_) cudaFree(kv.second);
  t64_.clear();
  t32_.clear();
}

const double2* TwiddleCache::get64(int L, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = t64_.find(L);
  if (it != t64_.end()) return it->second;
  std::vector<double> re, im;
  twiddle_host(L, re, im);
  std::vector<double2> h(L);
  for (int j = 0; j < L; ++j) h[j] = make_double2(re[j], im[j]);
  double2* d = nullptr;
  if (cudaMalloc(&d, sizeof(double2) * L) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h.data(), sizeof(double2) * L, cudaMemcpyHostToDevice) != cudaSuccess) { cudaFree(d); return nullptr; }
  t64_[L] = d;
  return d;
}

const float2* TwiddleCache::get32(int L, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = t32_.find(L);
  if (it != t32_.end()) return it->second;
  std::vector<double> re, im;
  twiddle_host(L, re, im);
  std::vector<float2> h(L);
  for (int j = 0; j < L; ++j) h[j] = make_float2((float)re[j], (float)im[j]);
  float2* d = nullptr;
  if (cudaMalloc(&d, sizeof(float2) * L) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h.data(), sizeof(float2) * L, cudaMemcpyHostToDevice) != cudaSuccess) { cudaFree(d); return nullptr; }
  t32_[L] = d;
  return d;
}

template <> const cplx<double>* TwiddleCache::get<double>(int L, cudaStream_t s) { return get64(L, s); }
template <> const cplx<float>* TwiddleCache::get<float>(int L, cudaStream_t s) { return get32(L, s); }

// ---------------------------------------------------------------------------
// 3D transforms (FourierTransformForward/Backward + ApplyNorm,
// src/grid_fft.cc:199-270): r2c = z, y, x passes; c2r = x, y, z passes
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t fft3d_r2c(mf_ctx* c, T* data, int n) {
  cudaStream_t s = c->stream;
  const int H = n / 2, Kz = H + 1;
  const cplx<T>* twH = c->tw.get<T>(H, s);
  const cplx<T>* twN = c->tw.get<T>(n, s);
  if (!twH || !twN) return cudaErrorMemoryAllocation;
  const T norm = T(1.0 / std::sqrt((double)n * (double)n * (double)n));
  cudaError_t e;
  {
    LaunchScope ls(c, KK_FFT_Z);
    e = Launch<T>::z_r2c_plain(H, PlainZOp<T>{data, n, T(1)}, n * n, Kz, twH, twN, s);
  }
  if (e != cudaSuccess) return e;
  cplx<T>* z = reinterpret_cast<cplx<T>*>(data);
  {
    LaunchScope ls(c, KK_FFT_COL);
    e = Launch<T>::colfft_plain(n, false, PlainStridedOp<T>{z, Kz, (long long)n * Kz, T(1)}, n, Kz, twN, s);
  }
  if (e != cudaSuccess) return e;
  LaunchScope ls(c, KK_FFT_COL);
  return Launch<T>::colfft_plain(n, false, PlainStridedOp<T>{z, (long long)n * Kz, Kz, norm}, n, Kz, twN, s);
}

template <typename T>
cudaError_t fft3d_c2r(mf_ctx* c, T* data, int n) {
  cudaStream_t s = c->stream;
  const int H = n / 2, Kz = H + 1;
  const cplx<T>* twH = c->tw.get<T>(H, s);
  const cplx<T>* twN = c->tw.get<T>(n, s);
  if (!twH || !twN) return cudaErrorMemoryAllocation;
  const T norm = T(1.0 / std::sqrt((double)n * (double)n * (double)n));
  cplx<T>* z = reinterpret_cast<cplx<T>*>(data);
  cudaError_t e;
  {
    LaunchScope ls(c, KK_FFT_COL);
    e = Launch<T>::colfft_plain(n, true, PlainStridedOp<T>{z, (long long)n * Kz, Kz, T(1)}, n, Kz, twN, s);
  }
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls(c, KK_FFT_COL);
    e = Launch<T>::colfft_plain(n, true, PlainStridedOp<T>{z, Kz, (long long)n * Kz, T(1)}, n, Kz, twN, s);
  }
  if (e != cudaSuccess) return e;
  LaunchScope ls(c, KK_FFT_Z);
  return Launch<T>::z_c2r_plain(H, PlainZOp<T>{data, n, norm}, n * n, Kz, twH, twN, s);
}

template cudaError_t fft3d_r2c<float>(mf_ctx*, float*, int);
template cudaError_t fft3d_r2c<double>(mf_ctx*, double*, int);
template cudaError_t fft3d_c2r<float>(mf_ctx*, float*, int);
template cudaError_t fft3d_c2r<double>(mf_ctx*, double*, int);

// ---------------------------------------------------------------------------
// convolution driver: x/y passes of the operands' c2r, fused z pass,
// y/x passes of the product's r2c with unpad + output operator
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t conv_run(mf_conv* cv, const Operand<T>* ops, int nop, cplx<T>* target, int out_op, T x,
                     int post_invlap) {
  mf_ctx* c = cv->ctx;
  cudaStream_t s = c->stream;
  const bool orszag = cv->kind == MF_CONV_ORSZAG;
  const int N = cv->n, M = orszag ? 3 * N / 2 : N, Kz = N / 2 + 1, H = M / 2;
  const ConvGeom g{N, M, Kz, orszag};
  const T kfac = T(2.0 * M_PI / cv->L);
  const double M3 = (double)M * M * M, N3 = (double)N * N * N;
  const T scale_in = orszag ? T(std::pow(1.5, 1.5) / std::sqrt(M3)) : T(1.0 / std::sqrt(N3));
  const T scale_out = orszag ? T(1.0 / std::sqrt(M3) / (std::sqrt(M3) / std::sqrt(N3))) : T(1.0 / std::sqrt(N3));
  const cplx<T>* twM = c->tw.get<T>(M, s);
  const cplx<T>* twH = c->tw.get<T>(H, s);
  if (!twM || !twH) return cudaErrorMemoryAllocation;
  const size_t per = (size_t)M * M * Kz;
  cplx<T>* B[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < nop; ++k) B[k] = reinterpret_cast<cplx<T>*>(cv->work) + k * per;

  ConvXInvOp<T> xo{};
  for (int k = 0; k < nop; ++k) { xo.opnd[k] = ops[k]; xo.dst[k] = B[k]; }
  xo.g = g;
  xo.kfac = kfac;
  xo.scale = scale_in;
  cudaError_t e;
  {
    LaunchScope ls(c, KK_CONV_XINV);
    e = Launch<T>::conv_xinv(M, xo, N, Kz, nop, twM, s);
  }
  if (e != cudaSuccess) return e;

  ConvYInvOp<T> yo{};
  for (int k = 0; k < nop; ++k) { yo.src[k] = B[k]; yo.dst[k] = B[k]; }
  yo.g = g;
  {
    LaunchScope ls(c, KK_CONV_YINV);
    e = Launch<T>::conv_yinv(M, yo, M, Kz, nop, twM, s);
  }
  if (e != cudaSuccess) return e;

  ZConvArgs<T> za{};
  for (int k = 0; k < nop; ++k) za.in[k] = B[k];
  za.out = B[nop - 1];
  za.nop = nop;
  za.kin = Kz;
  za.kout = Kz;
  za.in_stride = Kz;
  za.out_stride = Kz;
  za.nlines = M * M;
  za.out_scale = T(1);
  za.err = c->d_err;
  {
    LaunchScope ls(c, KK_CONV_Z);
    e = Launch<T>::z_conv(H, za, twH, twM, s);
  }
  if (e != cudaSuccess) return e;

  ConvYFwdOp<T> yf{B[nop - 1], B[nop - 1], g};
  {
    LaunchScope ls(c, KK_CONV_YFWD);
    e = Launch<T>::conv_yfwd(M, yf, M, Kz, twM, s);
  }
  if (e != cudaSuccess) return e;

  ConvXFwdOp<T> xf{};
  xf.src = B[nop - 1];
  xf.target = target;
  xf.g = g;
  xf.scale = scale_out;
  xf.out_op = out_op;
  xf.x = x;
  xf.post_invlap = post_invlap;
  xf.kfac = kfac;
  LaunchScope ls(c, KK_CONV_XFWD);
  return Launch<T>::conv_xfwd(M, xf, N, Kz, twM, s);
}

template cudaError_t conv_run<float>(mf_conv*, const Operand<float>*, int, cplx<float>*, int, float, int);
template cudaError_t conv_run<double>(mf_conv*, const Operand<double>*, int, cplx<double>*, int, double, int);

}  // namespace mf

using namespace mf;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" const char* mf_version(void) { return MF_VERSION_STR; }

extern "C" int mf_grid_size_supported(int n) { return grid_size_supported(n) ? 1 : 0; }

extern "C" int mf_ctx_create(int device, mf_ctx** out) {
  if (!out) return MF_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MF_ERR_CUDA;
  if (device < 0 || device >= ndev) return MF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MF_ERR_CUDA;
  mf_ctx* c = new (std::nothrow) mf_ctx();
  if (!c) return MF_ERR_OOM;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return MF_ERR_CUDA;
  }
  if (cudaMalloc(&c->d_err, sizeof(int)) != cudaSuccess || cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return MF_ERR_CUDA;
  }
  *out = c;
  return MF_OK;
}

extern "C" int mf_ctx_destroy(mf_ctx* c) {
  if (!c) return MF_ERR_ARG;
  if (c->children > 0)
    return set_err(c, MF_ERR_STATE, "mf_ctx_destroy: " + std::to_string(c->children) + " objects still alive on this context");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->tw.release();
  for (auto& rec : c->prof_events) { cudaEventDestroy(rec.second.first); cudaEventDestroy(rec.second.second); }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  cudaFree(c->d_err);
  cudaStreamDestroy(c->stream);
  delete c;
  return MF_OK;
}

extern "C" const char* mf_last_error(const mf_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int mf_ctx_synchronize(mf_ctx* c) {
  if (!c) return MF_ERR_ARG;
  cudaSetDevice(c->device);
  return check_device_error(c);
}

// ---------------------------------------------------------------------------
// grids
// ---------------------------------------------------------------------------
extern "C" int mf_grid_create(mf_ctx* c, int n, double boxlen, int prec, int space, mf_grid** out) {
  if (!c || !out) return MF_ERR_ARG;
  *out = nullptr;
  if (!grid_size_supported(n)) return set_err(c, MF_ERR_SHAPE, "mf_grid_create: unsupported grid size " + std::to_string(n));
  if (prec != MF_PREC_F64 && prec != MF_PREC_F32) return set_err(c, MF_ERR_ARG, "mf_grid_create: bad precision");
  if (space != MF_SPACE_R && space != MF_SPACE_K) return set_err(c, MF_ERR_ARG, "mf_grid_create: bad space");
  if (!(boxlen > 0)) return set_err(c, MF_ERR_ARG, "mf_grid_create: box length must be positive");
  cudaSetDevice(c->device);
  mf_grid* g = new (std::nothrow) mf_grid();
  if (!g) return MF_ERR_OOM;
  g->ctx = c;
  g->n = n;
  g->L = boxlen;
  g->prec = prec;
  g->space = space;
  g->bytes = grid_reals(n) * prec_size(prec);
  cudaError_t e = cudaMalloc(&g->d, g->bytes);
  if (e != cudaSuccess) {
    delete g;
    return cuda_err(c, e, "mf_grid_create: cudaMalloc");
  }
  ++c->children;
  *out = g;
  return MF_OK;
}

extern "C" int mf_grid_destroy(mf_grid* g) {
  if (!g) return MF_ERR_ARG;
  cudaSetDevice(g->ctx->device);
  cudaStreamSynchronize(g->ctx->stream);
  cudaFree(g->d);
  --g->ctx->children;
  delete g;
  return MF_OK;
}

extern "C" int mf_grid_info(const mf_grid* g, int* n, int* prec, int* space, void** dptr, size_t* bytes) {
  if (!g) return MF_ERR_ARG;
  if (n) *n = g->n;
  if (prec) *prec = g->prec;
  if (space) *space = g->space;
  if (dptr) *dptr = g->d;
  if (bytes) *bytes = g->bytes;
  return MF_OK;
}

extern "C" int mf_grid_upload(mf_grid* g, const void* host, int space) {
  if (!g || !host) return MF_ERR_ARG;
  if (space != MF_SPACE_R && space != MF_SPACE_K) return set_err(g->ctx, MF_ERR_ARG, "mf_grid_upload: bad space");
  mf_ctx* c = g->ctx;
  cudaSetDevice(c->device);
  cudaError_t e = cudaMemcpyAsync(g->d, host, g->bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_upload");
  g->space = space;
  return MF_OK;
}

extern "C" int mf_grid_download(mf_grid* g, void* host) {
  if (!g || !host) return MF_ERR_ARG;
  mf_ctx* c = g->ctx;
  cudaSetDevice(c->device);
  cudaError_t e = cudaMemcpyAsync(host, g->d, g->bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_err(c, e, "mf_grid_download");
}

extern "C" int mf_grid_fill_real64(mf_grid* g, const double* host) {
  if (!g || !host) return MF_ERR_ARG;
  mf_ctx* c = g->ctx;
  cudaSetDevice(c->device);
  const size_t n3 = (size_t)g->n * g->n * g->n;
  double* tmp = nullptr;
  cudaError_t e = cudaMallocAsync(&tmp, n3 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_fill_real64: alloc");
  e = cudaMemcpyAsync(tmp, host, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->d, 0, g->bytes, c->stream);
  if (e == cudaSuccess)
    e = (g->prec == MF_PREC_F64) ? pw_fill_from_f64<double>((double*)g->d, tmp, g->n, c->stream)
                                 : pw_fill_from_f64<float>((float*)g->d, tmp, g->n, c->stream);
  cudaFreeAsync(tmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_fill_real64");
  g->space = MF_SPACE_R;
  return MF_OK;
}

extern "C" int mf_grid_fft_forward(mf_grid* g, int do_transform) {
  if (!g) return MF_ERR_ARG;
  if (g->space == MF_SPACE_K) return MF_OK;
  mf_ctx* c = g->ctx;
  if (do_transform) {
    cudaSetDevice(c->device);
    cudaError_t e = (g->prec == MF_PREC_F64) ? fft3d_r2c<double>(c, (double*)g->d, g->n)
                                             : fft3d_r2c<float>(c, (float*)g->d, g->n);
    if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_fft_forward");
  }
  g->space = MF_SPACE_K;
  return MF_OK;
}

extern "C" int mf_grid_fft_backward(mf_grid* g, int do_transform) {
  if (!g) return MF_ERR_ARG;
  if (g->space == MF_SPACE_R) return MF_OK;
  mf_ctx* c = g->ctx;
  if (do_transform) {
    cudaSetDevice(c->device);
    cudaError_t e = (g->prec == MF_PREC_F64) ? fft3d_c2r<double>(c, (double*)g->d, g->n)
                                             : fft3d_c2r<float>(c, (float*)g->d, g->n);
    if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_fft_backward");
  }
  g->space = MF_SPACE_R;
  return MF_OK;
}

extern "C" int mf_grid_zero(mf_grid* g) {
  if (!g) return MF_ERR_ARG;
  cudaSetDevice(g->ctx->device);
  return cuda_err(g->ctx, cudaMemsetAsync(g->d, 0, g->bytes, g->ctx->stream), "mf_grid_zero");
}

extern "C" int mf_grid_scale(mf_grid* g, double x) {
  if (!g) return MF_ERR_ARG;
  cudaSetDevice(g->ctx->device);
  const size_t nr = grid_reals(g->n);
  LaunchScope ls(g->ctx, KK_POINTWISE);
  cudaError_t e = (g->prec == MF_PREC_F64) ? pw_scale<double>((double*)g->d, nr, x, g->ctx->stream)
                                           : pw_scale<float>((float*)g->d, nr, (float)x, g->ctx->stream);
  return cuda_err(g->ctx, e, "mf_grid_scale");
}

extern "C" int mf_grid_zero_dc(mf_grid* g) {
  if (!g) return MF_ERR_ARG;
  if (g->space != MF_SPACE_K) return set_err(g->ctx, MF_ERR_STATE, "mf_grid_zero_dc: real-space branch not supported on the device");
  cudaSetDevice(g->ctx->device);
  LaunchScope ls(g->ctx, KK_POINTWISE);
  cudaError_t e = (g->prec == MF_PREC_F64) ? pw_zero_dc<double>((double*)g->d, g->ctx->stream)
                                           : pw_zero_dc<float>((float*)g->d, g->ctx->stream);
  return cuda_err(g->ctx, e, "mf_grid_zero_dc");
}

// RNG_plugin::Fill_Grid (include/random_plugin.hh:37) with the project
// generator on the device; declared in monofonic_gb300_ic.h
extern "C" int mf_grid_fill_white_noise(mf_grid* g, uint64_t seed) {
  if (!g) return MF_ERR_ARG;
  if (g->n & 1) return set_err(g->ctx, MF_ERR_SHAPE, "mf_grid_fill_white_noise: odd grid size");
  cudaSetDevice(g->ctx->device);
  cudaError_t e;
  {
    LaunchScope ls(g->ctx, KK_POINTWISE);
    e = (g->prec == MF_PREC_F64) ? pw_white_noise<double>((double*)g->d, g->n, seed, nullptr, g->ctx->stream)
                                 : pw_white_noise<float>((float*)g->d, g->n, seed, nullptr, g->ctx->stream);
  }
  if (e != cudaSuccess) return cuda_err(g->ctx, e, "mf_grid_fill_white_noise");
  g->space = MF_SPACE_R;
  return MF_OK;
}

extern "C" int mf_grid_inverse_laplacian(mf_grid* g) {
  if (!g) return MF_ERR_ARG;
  int rc = mf_grid_fft_forward(g, 1);
  if (rc) return rc;
  const double kfac = 2.0 * M_PI / g->L;
  LaunchScope ls(g->ctx, KK_POINTWISE);
  cudaError_t e = (g->prec == MF_PREC_F64)
                      ? pw_invlap<double>((cplx<double>*)g->d, g->n, kfac, g->ctx->stream)
                      : pw_invlap<float>((cplx<float>*)g->d, g->n, kfac, g->ctx->stream);
  return cuda_err(g->ctx, e, "mf_grid_inverse_laplacian");
}

extern "C" int mf_grid_shift(mf_grid* g, const double s[3], int transform_back) {
  if (!g || !s) return MF_ERR_ARG;
  int rc = mf_grid_fft_forward(g, 1);
  if (rc) return rc;
  const double kfac = 2.0 * M_PI / g->L, dx = g->L / g->n;
  cudaError_t e = (g->prec == MF_PREC_F64)
                      ? pw_shift<double>((cplx<double>*)g->d, g->n, kfac, dx, s, g->ctx->stream)
                      : pw_shift<float>((cplx<float>*)g->d, g->n, kfac, dx, s, g->ctx->stream);
  if (e != cudaSuccess) return cuda_err(g->ctx, e, "mf_grid_shift");
  if (transform_back) return mf_grid_fft_backward(g, 1);
  return MF_OK;
}

extern "C" int mf_grid_power_spectrum(mf_grid* g, double* bin_k, double* bin_P, double* bin_eP, int64_t* bin_count,
                                      int nbins_cap, int* nbins_out) {
  if (!g || !nbins_out) return MF_ERR_ARG;
  mf_ctx* c = g->ctx;
  int rc = mf_grid_fft_forward(g, 1);
  if (rc) return rc;
  const double kfac = 2.0 * M_PI / g->L;
  const double kmax = kfac * (g->n / 2), kmin = kfac;
  const int nbins = (int)(kmax / kmin);
  *nbins_out = nbins;
  if (nbins_cap < nbins || !bin_k || !bin_P || !bin_eP || !bin_count)
    return set_err(c, MF_ERR_ARG, "mf_grid_power_spectrum: output arrays too small");
  double* acc = nullptr;
  cudaError_t e = cudaMallocAsync(&acc, sizeof(double) * 4 * nbins, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, sizeof(double) * 4 * nbins, c->stream);
  if (e == cudaSuccess)
    e = (g->prec == MF_PREC_F64) ? pw_power_spectrum<double>((cplx<double>*)g->d, g->n, kfac, nbins, acc, c->stream)
                                 : pw_power_spectrum<float>((cplx<float>*)g->d, g->n, kfac, nbins, acc, c->stream);
  std::vector<double> h(4 * (size_t)nbins);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), acc, sizeof(double) * 4 * nbins, cudaMemcpyDeviceToHost, c->stream);
  if (acc) cudaFreeAsync(acc, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_grid_power_spectrum");
  // normalisation (grid_fft.cc:1198-1209)
  const double volfac = g->L * g->L * g->L / std::pow(2.0 * M_PI, 3.0);
  const double fnorm = 1.0 / std::sqrt((double)g->n * g->n * g->n);
  const double fftfac = fnorm * fnorm;
  for (int i = 0; i < nbins; ++i) {
    const double cnt = h[3 * nbins + i];
    bin_count[i] = (int64_t)llround(cnt);
    bin_k[i] = h[2 * nbins + i];
    bin_P[i] = h[i];
    bin_eP[i] = h[nbins + i];
    if (cnt > 0) {
      bin_k[i] /= cnt;
      bin_P[i] = bin_P[i] / cnt * volfac * fftfac;
      bin_eP[i] = std::sqrt(bin_eP[i] / cnt - bin_P[i] * bin_P[i]) / std::sqrt(cnt) * volfac * fftfac;
    }
  }
  return MF_OK;
}

extern "C" int mf_grid_write_power_spectrum(mf_grid* g, const char* path) {
  if (!g || !path) return MF_ERR_ARG;
  const int cap = g->n;  // int(kmax / kmin) = n/2 bins
  std::vector<double> k(cap), P(cap), eP(cap);
  std::vector<int64_t> cnt(cap);
  int nb = 0;
  int rc = mf_grid_power_spectrum(g, k.data(), P.data(), eP.data(), cnt.data(), cap, &nb);
  if (rc) return rc;
  FILE* fp = std::fopen(path, "w");
  if (!fp) return set_err(g->ctx, MF_ERR_IO, std::string("mf_grid_write_power_spectrum: cannot create ") + path);
  // the reference streams with setw and the default float format (%g)
  bool ok = std::fprintf(fp, "# %14s%16s%16s%16s\n", "k", "P(k)", "err. P(k)", "#modes") > 0;
  for (int b = 0; b < nb && ok; ++b)
    if (cnt[b] > 0) ok = std::fprintf(fp, "%16g%16g%16g%16lld\n", k[b], P[b], eP[b], (long long)cnt[b]) > 0;
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? MF_OK : set_err(g->ctx, MF_ERR_IO, std::string("mf_grid_write_power_spectrum: write failed on ") + path);
}

// ---------------------------------------------------------------------------
// convolvers
// ---------------------------------------------------------------------------
extern "C" int mf_conv_create(mf_ctx* c, int n, double boxlen, int prec, int kind, mf_conv** out) {
  if (!c || !out) return MF_ERR_ARG;
  *out = nullptr;
  if (!grid_size_supported(n)) return set_err(c, MF_ERR_SHAPE, "mf_conv_create: unsupported grid size");
  if (kind != MF_CONV_ORSZAG && kind != MF_CONV_NAIVE) return set_err(c, MF_ERR_ARG, "mf_conv_create: bad kind");
  if (prec != MF_PREC_F64 && prec != MF_PREC_F32) return set_err(c, MF_ERR_ARG, "mf_conv_create: bad precision");
  cudaSetDevice(c->device);
  mf_conv* cv = new (std::nothrow) mf_conv();
  if (!cv) return MF_ERR_OOM;
  cv->ctx = c;
  cv->n = n;
  cv->L = boxlen;
  cv->prec = prec;
  cv->kind = kind;
  const int M = (kind == MF_CONV_ORSZAG) ? 3 * n / 2 : n;
  cv->nbuf = (kind == MF_CONV_ORSZAG) ? 2 : 3;
  cv->work_bytes = (size_t)cv->nbuf * M * M * (n / 2 + 1) * 2 * prec_size(prec);
  cudaError_t e = cudaMalloc(&cv->work, cv->work_bytes);
  if (e != cudaSuccess) {
    delete cv;
    return cuda_err(c, e, "mf_conv_create: work buffers");
  }
  if (kind == MF_CONV_ORSZAG) {
    int rc = mf_grid_create(c, n, boxlen, prec, MF_SPACE_K, &cv->fbuf);
    if (rc) {
      cudaFree(cv->work);
      delete cv;
      return rc;
    }
  }
  ++c->children;
  *out = cv;
  return MF_OK;
}

extern "C" int mf_conv_destroy(mf_conv* cv) {
  if (!cv) return MF_ERR_ARG;
  cudaSetDevice(cv->ctx->device);
  cudaStreamSynchronize(cv->ctx->stream);
  if (cv->fbuf) mf_grid_destroy(cv->fbuf);
  cudaFree(cv->work);
  --cv->ctx->children;
  delete cv;
  return MF_OK;
}

namespace {

int check_operand(mf_conv* cv, const mf_operand* o, const char* where) {
  if (!o || !o->grid) return set_err(cv->ctx, MF_ERR_ARG, std::string(where) + ": null operand");
  const mf_grid* g = o->grid;
  if (g->n != cv->n || g->prec != cv->prec)
    return set_err(cv->ctx, MF_ERR_SHAPE, std::string(where) + ": operand grid does not match the convolver");
  if (o->kind < MF_OPND_PLAIN || o->kind > MF_OPND_GRAD) return set_err(cv->ctx, MF_ERR_ARG, std::string(where) + ": bad operand kind");
  const int nd = (o->kind == MF_OPND_PLAIN) ? 0 : (o->kind == MF_OPND_GRAD) ? 1 : (o->kind == MF_OPND_HESS) ? 2 : 4;
  for (int i = 0; i < nd; ++i)
    if (o->d[i] < 0 || o->d[i] > 2) return set_err(cv->ctx, MF_ERR_ARG, std::string(where) + ": direction out of range");
  return MF_OK;
}

template <typename T>
Operand<T> to_operand(const mf_operand* o) {
  Operand<T> r{};
  r.f = reinterpret_cast<const cplx<T>*>(o->grid->d);
  r.kind = o->kind;
  for (int i = 0; i < 4; ++i) r.d[i] = o->d[i];
  return r;
}

template <typename T>
int conv_dispatch(mf_conv* cv, const mf_operand* const* ops, int nop, mf_grid* out, int op, double x, int invlap) {
  mf_ctx* c = cv->ctx;
  Operand<T> o[3];
  for (int k = 0; k < nop; ++k) o[k] = to_operand<T>(ops[k]);
  cudaError_t e;
  if (nop == 3 && cv->kind == MF_CONV_ORSZAG) {
    // convolve3: convolve2(kf1, kf2 -> fbuf_), then convolve2(fbuf_, kf3 -> op)
    e = conv_run<T>(cv, o, 2, reinterpret_cast<cplx<T>*>(cv->fbuf->d), OUT_ASSIGN, T(1), 0);
    if (e != cudaSuccess) return cuda_err(c, e, "convolve3 stage 1");
    Operand<T> o2[2];
    o2[0].f = reinterpret_cast<const cplx<T>*>(cv->fbuf->d);
    o2[0].kind = OPND_PLAIN;
    o2[1] = o[2];
    e = conv_run<T>(cv, o2, 2, reinterpret_cast<cplx<T>*>(out->d), op, T(x), invlap);
  } else {
    e = conv_run<T>(cv, o, nop, reinterpret_cast<cplx<T>*>(out->d), op, T(x), invlap);
  }
  return cuda_err(c, e, "convolve");
}

int conv_entry(mf_conv* cv, const mf_operand* const* ops, int nop, mf_grid* out, int op, double x, int invlap) {
  if (!cv || !out) return MF_ERR_ARG;
  mf_ctx* c = cv->ctx;
  for (int k = 0; k < nop; ++k) {
    int rc = check_operand(cv, ops[k], "convolve");
    if (rc) return rc;
  }
  if (out->n != cv->n || out->prec != cv->prec) return set_err(c, MF_ERR_SHAPE, "convolve: output grid does not match");
  if (op < MF_OP_ASSIGN || op > MF_OP_AXPY) return set_err(c, MF_ERR_ARG, "convolve: bad output operator");
  cudaSetDevice(c->device);
  // transform to Fourier space in case fields are not (convolution.hh:149-151)
  for (int k = 0; k < nop; ++k) {
    int rc = mf_grid_fft_forward(ops[k]->grid, 1);
    if (rc) return rc;
  }
  // the output is written in k-space; assign needs no prior content
  if (op == MF_OP_ASSIGN) out->space = MF_SPACE_K;
  else if (out->space != MF_SPACE_K) {
    int rc = mf_grid_fft_forward(out, 1);
    if (rc) return rc;
  }
  int rc = (cv->prec == MF_PREC_F64) ? conv_dispatch<double>(cv, ops, nop, out, op, x, invlap)
                                     : conv_dispatch<float>(cv, ops, nop, out, op, x, invlap);
  if (rc == MF_OK) out->space = MF_SPACE_K;
  return rc;
}

}  // namespace

extern "C" int mf_conv_convolve2(mf_conv* cv, const mf_operand* a, const mf_operand* b, mf_grid* out, int op, double x) {
  const mf_operand* ops[2] = {a, b};
  return conv_entry(cv, ops, 2, out, op, x, 0);
}

extern "C" int mf_conv_convolve2_invlap(mf_conv* cv, const mf_operand* a, const mf_operand* b, mf_grid* out, int op,
                                        double x) {
  const mf_operand* ops[2] = {a, b};
  return conv_entry(cv, ops, 2, out, op, x, 1);
}

extern "C" int mf_conv_convolve3(mf_conv* cv, const mf_operand* a, const mf_operand* b, const mf_operand* c3,
                                 mf_grid* out, int op, double x) {
  const mf_operand* ops[3] = {a, b, c3};
  return conv_entry(cv, ops, 3, out, op, x, 0);
}

// ---------------------------------------------------------------------------
// measurement hooks
// ---------------------------------------------------------------------------
extern "C" int mf_ctx_stream(mf_ctx* c, void** stream) {
  if (!c || !stream) return MF_ERR_ARG;
  *stream = (void*)c->stream;
  return MF_OK;
}

extern "C" int mf_ctx_launch_counts(const mf_ctx* c, int64_t* counts, int n) {
  if (!c || !counts) return MF_ERR_ARG;
  for (int k = 0; k < n && k < KK_COUNT; ++k) counts[k] = c->launches[k];
  return MF_OK;
}

extern "C" int mf_ctx_profile(mf_ctx* c, int enable) {
  if (!c) return MF_ERR_ARG;
  c->profile = enable != 0;
  return MF_OK;
}

extern "C" int mf_ctx_profile_read(mf_ctx* c, double* ms, int64_t* counts, int n) {
  if (!c || !ms || !counts) return MF_ERR_ARG;
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_ctx_profile_read");
  for (int k = 0; k < n; ++k) { ms[k] = 0; counts[k] = 0; }
  for (auto& rec : c->prof_events) {
    float t = 0;
    if (cudaEventElapsedTime(&t, rec.second.first, rec.second.second) == cudaSuccess && rec.first < n) {
      ms[rec.first] += t;
      counts[rec.first] += 1;
    } else {
      cudaGetLastError();  // an unrecorded pair is skipped, not left for the next call to report
    }
    c->event_pool.push_back(rec.second.first);
    c->event_pool.push_back(rec.second.second);
  }
  c->prof_events.clear();
  return MF_OK;
}

// ---------------------------------------------------------------------------
// page-locked host buffers.  A buffer of at least one transparent huge page
// is an anonymous private mapping aligned to the kernel's PMD page size,
// advised MADV_HUGEPAGE, first-touched and then registered with the driver:
// the device reaches it through a few large translations.  On the GB300 host
// link, buffers of base pages (cudaHostAlloc, or malloc + cudaHostRegister)
// had whole copies drop from 193 GB/s (device to host) and 211 GB/s (host to
// device) to 12-60 GB/s at irregular times, while huge-page buffers kept the
// full rate.  Smaller buffers, and hosts without transparent huge pages, use
// cudaHostAlloc.
// ---------------------------------------------------------------------------
namespace {
struct HostMapping {
  void* base;
  size_t len;
};
std::mutex g_host_mu;
std::unordered_map<void*, HostMapping> g_host_maps;

// PMD huge page size when transparent huge pages can be requested, else 0
size_t thp_bytes() {
  static const size_t sz = [] {
    unsigned long long v = 0;
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
      if (std::fscanf(f, "%llu", &v) != 1) v = 0;
      std::fclose(f);
    }
    char mode[128] = {0};
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/enabled", "r")) {
      if (!std::fgets(mode, sizeof mode, f)) mode[0] = 0;
      std::fclose(f);
    }
    if (!std::strstr(mode, "[always]") && !std::strstr(mode, "[madvise]")) v = 0;
    return (size_t)v;
  }();
  return sz;
}

void* thp_alloc(size_t bytes) {
  const size_t hp = thp_bytes();
  if (!hp || bytes < hp) return nullptr;
  const size_t len = (bytes + hp - 1) / hp * hp;
  char* raw = (char*)mmap(nullptr, len + hp, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw == MAP_FAILED) return nullptr;
  char* a = (char*)(((uintptr_t)raw + hp - 1) / hp * hp);
  if (a > raw) munmap(raw, (size_t)(a - raw));  // trim the alignment slack
  if (a + len < raw + len + hp) munmap(a + len, (size_t)(raw + len + hp - (a + len)));
  madvise(a, len, MADV_HUGEPAGE);
  madvise(a, len, MADV_DONTFORK);  // a child process must not share the registered pages copy-on-write
  std::memset(a, 0, len);          // first touch: faulted in as huge pages
  if (cudaHostRegister(a, len, cudaHostRegisterPortable) != cudaSuccess) {
    cudaGetLastError();
    munmap(a, len);
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_maps[a] = HostMapping{a, len};
  return a;
}
}  // namespace

extern "C" int mf_host_alloc(size_t bytes, void** out) {
  if (!out) return MF_ERR_ARG;
  *out = thp_alloc(bytes);
  if (*out) return MF_OK;
  if (cudaHostAlloc(out, bytes, cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return MF_ERR_OOM;
  }
  return MF_OK;
}

extern "C" int mf_host_free(void* p) {
  if (!p) return MF_OK;
  HostMapping m{nullptr, 0};
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_maps.find(p);
    if (it != g_host_maps.end()) {
      m = it->second;
      g_host_maps.erase(it);
    }
  }
  if (m.base) {
    cudaHostUnregister(m.base);
    munmap(m.base, m.len);
  } else {
    cudaFreeHost(p);
  }
  return MF_OK;
}

extern "C" int mf_host_huge_page_bytes(size_t* bytes) {
  if (!bytes) return MF_ERR_ARG;
  *bytes = thp_bytes();
  return MF_OK;
}

extern "C" int mf_copy_to_host(void* host, const void* device, size_t bytes) {
  if (bytes && (!host || !device)) return MF_ERR_ARG;
  return cudaMemcpy(host, device, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}
