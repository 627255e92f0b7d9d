// Allocation-free Orszag convolution entry point.
//
// Some callers cannot allocate device memory: an N-body or hydro code that
// runs the initial-condition generator in-process usually hands the whole
// device to its own memory pool, and latency-sensitive host code may not be
// allowed the implicit device synchronisation of cudaMalloc/cudaFree.  For
// them mf_conv_convolve2_noalloc performs one Orszag 3/2 convolve2 without any
// allocation: the padded work buffers live in a fixed file-scope device array
// (kScratchBytes, held by every GPU that loads the library until the process
// exits) and the twiddle tables in small file-scope device arrays.
//
// The device addresses of those arrays are looked up once per device with
// cudaGetSymbolAddress (in host code an array's name is only a host-side
// stand-in) during the first call on that device; that first call should
// therefore come before any stream capture.  Every call shares the one
// scratch array and leaves its contents behind; nothing in it has to start at
// zero except the wait-timeout flag, which each call clears.  Calls whose work
// overlaps on the GPU (different streams or host threads) race on the shared
// scratch and must be serialised by the caller.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "mf_runtime.h"

namespace {

using namespace mf;

// 48 MiB: Orszag convolve2 up to N = 128 in FP32 (38.3 MB) and N = 96 in FP64 (32.5 MB)
constexpr size_t kScratchBytes = size_t(48) << 20;
// twiddle lengths of the supported sizes: M = 3N/2 and M/2 for N in {16,32,64,96,128}
constexpr int kTwLens[] = {12, 24, 48, 72, 96, 144, 192};
constexpr int kNumTw = sizeof(kTwLens) / sizeof(kTwLens[0]);
constexpr int kTwTotal = 12 + 24 + 48 + 72 + 96 + 144 + 192;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static __device__ __align__(256) double2 g_tw64[kTwTotal];
static __device__ __align__(256) float2 g_tw32[kTwTotal];
static __device__ int g_err;

struct DeviceState {
  unsigned char* scratch = nullptr;
  double2* tw64 = nullptr;
  float2* tw32 = nullptr;
  int* err = nullptr;
};

std::mutex g_mu;
std::map<int, DeviceState> g_dev;

int tw_offset(int L) {
  int off = 0;
  for (int i = 0; i < kNumTw; ++i) {
    if (kTwLens[i] == L) return off;
    off += kTwLens[i];
  }
  return -1;
}

// set-up for the current device: symbol addresses and twiddle tables
int setup_device(int dev, DeviceState* out, std::string* why) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_dev.find(dev);
  if (it != g_dev.end()) {
    *out = it->second;
    return MF_OK;
  }
  DeviceState st;
  cudaError_t e = cudaGetSymbolAddress((void**)&st.scratch, g_scratch);
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&st.tw64, g_tw64);
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&st.tw32, g_tw32);
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&st.err, g_err);
  if (e != cudaSuccess) {
    *why = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return MF_ERR_CUDA;
  }
  std::vector<double2> h64(kTwTotal);
  std::vector<float2> h32(kTwTotal);
  const long double pi = 3.141592653589793238462643383279502884L;
  int off = 0;
  for (int i = 0; i < kNumTw; ++i) {
    const int L = kTwLens[i];
    for (int j = 0; j < L; ++j) {
      double re = (double)cosl(2.0L * pi * j / L), im = (double)(-sinl(2.0L * pi * j / L));
      if ((4 * j) % L == 0) {
        const int q = (4 * j) / L;
        const double c[4] = {1, 0, -1, 0}, s[4] = {0, -1, 0, 1};
        re = c[q];
        im = s[q];
      }
      h64[off + j] = make_double2(re, im);
      h32[off + j] = make_float2((float)re, (float)im);
    }
    off += L;
  }
  e = cudaMemcpyToSymbol(g_tw64, h64.data(), sizeof(double2) * kTwTotal);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tw32, h32.data(), sizeof(float2) * kTwTotal);
  if (e != cudaSuccess) {
    *why = std::string("twiddle upload: ") + cudaGetErrorString(e);
    return MF_ERR_CUDA;
  }
  g_dev[dev] = st;
  *out = st;
  return MF_OK;
}

template <typename T>
const cplx<T>* tw_table(const DeviceState& st, int L);
template <>
const cplx<double>* tw_table<double>(const DeviceState& st, int L) { return st.tw64 + tw_offset(L); }
template <>
const cplx<float>* tw_table<float>(const DeviceState& st, int L) { return st.tw32 + tw_offset(L); }

// the five passes of the Orszag convolve2, work buffers in the static scratch
template <typename T>
cudaError_t conv2_static(const DeviceState& st, cudaStream_t s, int N, double boxlen, const Operand<T>* ops,
                         cplx<T>* target, int out_op, T x) {
  const int M = 3 * N / 2, Kz = N / 2 + 1, H = M / 2;
  const ConvGeom g{N, M, Kz, true};
  const T kfac = T(2.0 * M_PI / boxlen);
  const double M3 = (double)M * M * M, N3 = (double)N * N * N;
  const T scale_in = T(std::pow(1.5, 1.5) / std::sqrt(M3));
  const T scale_out = T(1.0 / std::sqrt(M3) / (std::sqrt(M3) / std::sqrt(N3)));
  const cplx<T>* twM = tw_table<T>(st, M);
  const cplx<T>* twH = tw_table<T>(st, H);
  const size_t per = (size_t)M * M * Kz;
  cplx<T>* B0 = reinterpret_cast<cplx<T>*>(st.scratch);
  cplx<T>* B1 = B0 + per;

  ConvXInvOp<T> xo{};
  xo.opnd[0] = ops[0];
  xo.opnd[1] = ops[1];
  xo.dst[0] = B0;
  xo.dst[1] = B1;
  xo.g = g;
  xo.kfac = kfac;
  xo.scale = scale_in;
  cudaError_t e = Launch<T>::conv_xinv(M, xo, N, Kz, 2, twM, s);
  if (e != cudaSuccess) return e;
  ConvYInvOp<T> yo{};
  yo.src[0] = B0;
  yo.src[1] = B1;
  yo.dst[0] = B0;
  yo.dst[1] = B1;
  yo.g = g;
  e = Launch<T>::conv_yinv(M, yo, M, Kz, 2, twM, s);
  if (e != cudaSuccess) return e;
  ZConvArgs<T> za{};
  za.in[0] = B0;
  za.in[1] = B1;
  za.out = B1;
  za.nop = 2;
  za.kin = Kz;
  za.kout = Kz;
  za.in_stride = Kz;
  za.out_stride = Kz;
  za.nlines = M * M;
  za.out_scale = T(1);
  za.err = st.err;
  e = Launch<T>::z_conv(H, za, twH, twM, s);
  if (e != cudaSuccess) return e;
  ConvYFwdOp<T> yf{B1, B1, g};
  e = Launch<T>::conv_yfwd(M, yf, M, Kz, twM, s);
  if (e != cudaSuccess) return e;
  ConvXFwdOp<T> xf{};
  xf.src = B1;
  xf.target = target;
  xf.g = g;
  xf.scale = scale_out;
  xf.out_op = out_op;
  xf.x = x;
  xf.post_invlap = 0;
  xf.kfac = kfac;
  return Launch<T>::conv_xfwd(M, xf, N, Kz, twM, s);
}

int check_operand_kind(int kind, const int* d) {
  if (kind < MF_OPND_PLAIN || kind > MF_OPND_GRAD) return MF_ERR_ARG;
  const int nd = (kind == MF_OPND_PLAIN) ? 0 : (kind == MF_OPND_GRAD) ? 1 : (kind == MF_OPND_HESS) ? 2 : 4;
  for (int i = 0; i < nd; ++i)
    if (!d || d[i] < 0 || d[i] > 2) return MF_ERR_ARG;
  return MF_OK;
}

}  // namespace

extern "C" int mf_conv_convolve2_noalloc(void* stream, int n, double boxlen, int prec, const void* field_a,
                                         int kind_a, const int* dirs_a, const void* field_b, int kind_b,
                                         const int* dirs_b, void* out, int op, double x) {
  if (!field_a || !field_b || !out) return MF_ERR_ARG;
  if (prec != MF_PREC_F64 && prec != MF_PREC_F32) return MF_ERR_ARG;
  if (op < MF_OP_ASSIGN || op > MF_OP_AXPY) return MF_ERR_ARG;
  if (!(boxlen > 0)) return MF_ERR_ARG;
  if (check_operand_kind(kind_a, dirs_a) || check_operand_kind(kind_b, dirs_b)) return MF_ERR_ARG;
  if (n != 16 && n != 32 && n != 64 && n != 96 && n != 128) return MF_ERR_SHAPE;
  const int M = 3 * n / 2;
  const size_t need = (size_t)2 * M * M * (n / 2 + 1) * 2 * (prec == MF_PREC_F32 ? 4 : 8);
  if (need > kScratchBytes) return MF_ERR_SHAPE;  // beyond the static scratch (48 MiB)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MF_ERR_CUDA;
  DeviceState st;
  std::string why;
  int rc = setup_device(dev, &st, &why);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(st.err, 0, sizeof(int), s);
  if (e != cudaSuccess) return MF_ERR_CUDA;
  if (prec == MF_PREC_F64) {
    Operand<double> o[2];
    o[0].f = (const double2*)field_a;
    o[0].kind = kind_a;
    o[1].f = (const double2*)field_b;
    o[1].kind = kind_b;
    for (int i = 0; i < 4; ++i) {
      o[0].d[i] = dirs_a ? dirs_a[i] : 0;
      o[1].d[i] = dirs_b ? dirs_b[i] : 0;
    }
    e = conv2_static<double>(st, s, n, boxlen, o, (double2*)out, op, x);
  } else {
    Operand<float> o[2];
    o[0].f = (const float2*)field_a;
    o[0].kind = kind_a;
    o[1].f = (const float2*)field_b;
    o[1].kind = kind_b;
    for (int i = 0; i < 4; ++i) {
      o[0].d[i] = dirs_a ? dirs_a[i] : 0;
      o[1].d[i] = dirs_b ? dirs_b[i] : 0;
    }
    e = conv2_static<float>(st, s, n, boxlen, o, (float2*)out, op, (float)x);
  }
  if (e != cudaSuccess) return (e == cudaErrorMemoryAllocation) ? MF_ERR_OOM : MF_ERR_CUDA;
  // the call returns once the result is complete, so a bounded wait that ran
  // out inside the pipelined pass can be reported
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return MF_ERR_CUDA;
  int flag = 0;
  e = cudaMemcpy(&flag, st.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return MF_ERR_CUDA;
  return flag ? MF_ERR_TIMEOUT : MF_OK;
}
