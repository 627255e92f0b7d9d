// Pointwise k-space / real-space kernels on N-grids (padded in-place layout).
#include <cmath>
#include <type_traits>

#include "mf_noise.h"
#include "mf_tma.cuh"
#include "mf_runtime.h"

namespace mf {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(size_t n, int per = 1) {
  size_t b = (n + (size_t)kThreads * per - 1) / ((size_t)kThreads * per);
  if (b > 152u * 64u) b = 152u * 64u;
  if (b == 0) b = 1;
  return (unsigned)b;
}

template <typename T>
__global__ void k_scale(T* d, size_t n, T x) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) d[i] *= x;
}

template <typename T>
__global__ void k_zero_dc(T* d) {
  if (threadIdx.x == 0 && blockIdx.x == 0) { d[0] = T(0); d[1] = T(0); }
}

// apply_InverseLaplacian (grid_fft.hh:440-449): -x/k^2, then zero_DC_mode
template <typename T>
__global__ void k_invlap(cplx<T>* d, int n, T kfac) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const T kx = kcomp<T>(i, n, kfac), ky = kcomp<T>(j, n, kfac), kk = kcomp<T>(kz, n, kfac);
    const T k2 = kx * kx + ky * ky + kk * kk;
    cplx<T> v = d[idx];
    d[idx] = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(-v.x / k2, -v.y / k2);
  }
}

// white noise of the project RNG plugin on the device (the generator of
// mf_noise.h, the same bits as the host plugin), written into the padded
// real layout; pair p = cells 2p, 2p+1 of one z row (n even).  The seed is
// read from device memory when seed_dev is given (replayable graphs).
template <typename T>
__global__ void k_white_noise(T* d, int n, unsigned long long seed, const unsigned long long* seed_dev) {
  using T2 = typename cplx_of<T>::type;
  const unsigned long long sd = seed_dev ? *seed_dev : seed;
  const unsigned hn = (unsigned)n >> 1;
  const unsigned long long npair = (unsigned long long)n * n * hn;
  for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < npair;
       p += (unsigned long long)gridDim.x * blockDim.x) {
    double z0, z1;
    noise::normal_pair(p, sd, &z0, &z1);
    const unsigned long long line = p / hn;
    const unsigned k = 2u * (unsigned)(p - line * hn);
    T2 v;
    v.x = (T)z0;
    v.y = (T)z1;
    *reinterpret_cast<T2*>(d + line * (unsigned long long)(n + 2) + k) = v;
  }
}

// shift_field's phase (grid_fft.hh:835-838): x * exp(i (s.k) dx)
template <typename T>
__global__ void k_shift(cplx<T>* d, int n, T kfac, T dx, T s0, T s1, T s2) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const T sh = s0 * kcomp<T>(i, n, kfac) * dx + s1 * kcomp<T>(j, n, kfac) * dx + s2 * kcomp<T>(kz, n, kfac) * dx;
    T sn, cs;
    if constexpr (sizeof(T) == 4) sincosf(sh, &sn, &cs); else sincos(sh, &sn, &cs);
    d[idx] = cmul(d[idx], mkc<T>(cs, sn));
  }
}

template <typename T>
__global__ void k_fill_from_f64(T* d, const double* src, int n) {
  const size_t tot = (size_t)n * n * n;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < tot; c += (size_t)gridDim.x * blockDim.x) {
    const size_t line = c / n;
    const int k = (int)(c % n);
    d[line * (n + 2) + k] = T(src[c]);
  }
}

// binned |delta_k|^2 (grid_fft.cc:1133-1181): per-block shared histograms
template <typename T>
__global__ void k_pk(const cplx<T>* d, int n, double kfac, int nbins, double* acc) {
  extern __shared__ double sh[];  // 4 * nbins
  for (int b = threadIdx.x; b < 4 * nbins; b += blockDim.x) sh[b] = 0.0;
  __syncthreads();
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  const double kmin = kfac, kmax = kfac * (n / 2), dk = kmin;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const double kx = kcomp<double>(i, n, kfac), ky = kcomp<double>(j, n, kfac), kk = kcomp<double>(kz, n, kfac);
    // |k| without contraction into FMAs (modes of integer norm sit on bin
    // edges, so the bin follows the exact rounding of x*x + y*y + z*z)
    const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kk, kk)));
    if (k >= kmin && k < kmax) {
      const int b = (int)(k / dk);
      const cplx<T> z = d[idx];
      const double v = (double)z.x * (double)z.x + (double)z.y * (double)z.y;
      const double w = (kz == 0) ? 1.0 : 2.0;
      atomicAdd(&sh[b], w * v);
      atomicAdd(&sh[nbins + b], w * v * v);
      atomicAdd(&sh[2 * nbins + b], w * k);
      atomicAdd(&sh[3 * nbins + b], w);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 4 * nbins; b += blockDim.x)
    if (sh[b] != 0.0) atomicAdd(&acc[b], sh[b]);
}

}  // namespace

template <typename T>
cudaError_t pw_scale(T* d, size_t nreal, T x, cudaStream_t s) {
  k_scale<T><<<grid_for(nreal, 4), kThreads, 0, s>>>(d, nreal, x);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_zero_dc(T* d, cudaStream_t s) {
  k_zero_dc<T><<<1, 32, 0, s>>>(d);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_invlap(cplx<T>* d, int n, double kfac, cudaStream_t s) {
  k_invlap<T><<<grid_for((size_t)n * n * (n / 2 + 1), 4), kThreads, 0, s>>>(d, n, T(kfac));
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_shift(cplx<T>* d, int n, double kfac, double dx, const double sh[3], cudaStream_t s) {
  k_shift<T><<<grid_for((size_t)n * n * (n / 2 + 1), 4), kThreads, 0, s>>>(d, n, T(kfac), T(dx), T(sh[0]), T(sh[1]),
                                                                          T(sh[2]));
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_fill_from_f64(T* d, const double* src, int n, cudaStream_t s) {
  k_fill_from_f64<T><<<grid_for((size_t)n * n * n, 4), kThreads, 0, s>>>(d, src, n);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_white_noise(T* d, int n, unsigned long long seed, const unsigned long long* seed_dev, cudaStream_t s) {
  if (n <= 0 || (n & 1)) return cudaErrorInvalidValue;
  k_white_noise<T><<<grid_for((size_t)n * n * (n / 2), 2), kThreads, 0, s>>>(d, n, seed, seed_dev);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pw_power_spectrum(const cplx<T>* d, int n, double kfac, int nbins, double* acc, cudaStream_t s) {
  const size_t smem = (size_t)4 * nbins * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_pk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_pk<T><<<grid_for((size_t)n * n * (n / 2 + 1), 8), kThreads, smem, s>>>(d, n, kfac, nbins, acc);
  return cudaGetLastError();
}

#define INST(T)                                                                                      \
  template cudaError_t pw_scale<T>(T*, size_t, T, cudaStream_t);                                     \
  template cudaError_t pw_zero_dc<T>(T*, cudaStream_t);                                              \
  template cudaError_t pw_invlap<T>(cplx<T>*, int, double, cudaStream_t);                            \
  template cudaError_t pw_shift<T>(cplx<T>*, int, double, double, const double*, cudaStream_t);      \
  template cudaError_t pw_fill_from_f64<T>(T*, const double*, int, cudaStream_t);                    \
  template cudaError_t pw_white_noise<T>(T*, int, unsigned long long, const unsigned long long*, cudaStream_t); \
  template cudaError_t pw_power_spectrum<T>(const cplx<T>*, int, double, int, double*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace mf

// ---------------------------------------------------------------------------
// FMA-rate probe: 8 independent FMA chains per thread, used to measure the
// FP64 (and FP32) arithmetic ceiling of the device the pipeline runs on
// ---------------------------------------------------------------------------
namespace {
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
  T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const T r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (r == T(-12345.678)) out[0] = r;  // keeps the chains live
}
}  // namespace

extern "C" int mf_probe_fma_rate(mf_ctx* c, int prec, double* tflops) {
  if (!c || !tflops) return MF_ERR_ARG;
  cudaSetDevice(c->device);
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
  const int blocks = nsm * 8, threads = 256, iters = (prec == MF_PREC_F64) ? 2048 : 65536;
  void* out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, 16) != cudaSuccess) return MF_ERR_OOM;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, c->stream);
    if (prec == MF_PREC_F64)
      k_fma_probe<double><<<blocks, threads, 0, c->stream>>>((double*)out, iters, 0.999999, 1e-7);
    else
      k_fma_probe<float><<<blocks, threads, 0, c->stream>>>((float*)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return mf::cuda_err(c, e, "mf_probe_fma_rate");
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return MF_OK;
}

// ---------------------------------------------------------------------------
// bounded-wait self-test: the failure path of every TMA-pipelined kernel
// (mbar_wait_bounded) exercised without a fault.  One thread initialises an
// mbarrier expecting one arrival; nothing arrives and no copy is issued, so
// the phase never completes and the wait gives up after `polls` tries, sets
// the context's error flag and returns.
// ---------------------------------------------------------------------------
namespace {
__global__ void k_wait_selftest(int* err, long polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mf::mbar_init(&bar, 1);
    mf::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mf::mbar_wait_bounded_n(&bar, 0, err, 1, polls);
}
}  // namespace

extern "C" int mf_selftest_bounded_wait(mf_ctx* c, long polls) {
  if (!c) return MF_ERR_ARG;
  if (polls < 1 || polls > (1L << 24)) return mf::set_err(c, MF_ERR_ARG, "mf_selftest_bounded_wait: polls out of range");
  cudaSetDevice(c->device);
  k_wait_selftest<<<1, 32, 0, c->stream>>>(c->d_err, polls);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mf::cuda_err(c, e, "mf_selftest_bounded_wait");
  return mf::check_device_error(c);
}

// ---------------------------------------------------------------------------
// float-pair self-test: the FP32-bulk form carries the growth-weighted order
// sum (k_phitot) and the lattice positions q + Psi (lattice readout) as float
// pairs instead of FP64.  This kernel runs the same device helpers (ff_axpy,
// ff_add_q) on `count` pseudo-random inputs shaped like the pipeline's
// (three FP32 order terms with FP64 growth weights of z_start = 24; q a
// lattice coordinate times the box length, Psi an FP32 displacement) and
// counts the stored floats that differ from the FP64 evaluation rounded once.
// ---------------------------------------------------------------------------
namespace {
__device__ __forceinline__ uint64_t sm64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ float unit_f(uint64_t h) {  // uniform in (-1, 1), 24 random bits
  return ((float)(h >> 40) + 0.5f) * (1.0f / 8388608.0f) - 1.0f;
}
__global__ void k_float_pair_selftest(long long count, uint64_t seed, double w1, double w2, double w3, double L,
                                      int n, unsigned long long* mism) {
  float wh[3], wl[3];
  const double wd[3] = {w1, w2, w3};
  for (int q = 0; q < 3; ++q) {
    wh[q] = __double2float_rn(wd[q]);
    wl[q] = __double2float_rn(wd[q] - (double)wh[q]);
  }
  unsigned long long ms = 0, mq = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t h0 = sm64(seed ^ (uint64_t)i), h1 = sm64(h0), h2 = sm64(h1), h3 = sm64(h2), h4 = sm64(h3);
    // order sum: potentials of three orders with decreasing magnitudes
    const float a1 = unit_f(h0) * 1e3f, a2 = unit_f(h1) * 10.0f, a3 = unit_f(h2) * 0.1f;
    float rh = 0.f, rl = 0.f;
    mf::ff_axpy(wh[0], wl[0], a1, rh, rl);
    mf::ff_axpy(wh[1], wl[1], a2, rh, rl);
    mf::ff_axpy(wh[2], wl[2], a3, rh, rl);
    const float ff = rh + rl;
    const float dd = __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(w1, (double)a1), __dmul_rn(w2, (double)a2)),
                                                 __dmul_rn(w3, (double)a3)));
    ms += (ff != dd);
    // q + Psi: q = (idx + s) / n * L with s in {0, 1/4, 1/2}, as a float pair
    const int idx = (int)(h3 % (uint64_t)n);
    const double s = 0.25 * (double)((h3 >> 32) % 3u);
    const double q = __dmul_rn(__ddiv_rn((double)idx + s, (double)n), L);
    const float qh = __double2float_rn(q);
    const float2 qf = make_float2(qh, __double2float_rn(q - (double)qh));
    const float psi = unit_f(h4) * 5.0f;
    mq += (mf::ff_add_q(qf, psi) != __double2float_rn(__dadd_rn(q, (double)psi)));
  }
  if (ms) atomicAdd(&mism[0], ms);
  if (mq) atomicAdd(&mism[1], mq);
}
}  // namespace

extern "C" int mf_selftest_float_pairs(mf_ctx* c, long long count, uint64_t seed, double Dplus, long long* mism_sum,
                                       long long* mism_q) {
  if (!c || count < 1 || !mism_sum || !mism_q) return MF_ERR_ARG;
  cudaSetDevice(c->device);
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return mf::set_err(c, MF_ERR_OOM, "mf_selftest_float_pairs");
  cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c->stream);
  const double w1 = -Dplus, w2 = -3.0 / 7.0 * Dplus * Dplus, w3 = Dplus * Dplus * Dplus / 3.0;
  k_float_pair_selftest<<<152 * 8, 256, 0, c->stream>>>(count, seed, w1, w2, w3, 1000.0, 512, d);
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return mf::cuda_err(c, e, "mf_selftest_float_pairs");
  *mism_sum = (long long)h[0];
  *mism_q = (long long)h[1];
  return MF_OK;
}
