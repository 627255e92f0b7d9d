// Semiclassical (propagator perturbation theory, PPT) Eulerian fields of a
// species (ic_generator.cc:679-791): the wave function
//   psi = sqrt(1 + C delta_bc) exp(i (phi + phi2) / (hbar D+))
// drifted one step in k-space, the density |psi|^2 - 1 and the velocity
// hbar Im(conj(psi) grad psi) / (1 + rho).  Complex fields and their 3D
// complex-to-complex transforms run in FP64 whatever the pipeline precision:
// the density is a small difference of |psi|^2 and 1, and the phases reach
// hundreds of radians.
#include <cmath>
#include <cstdint>

#include "mf_ppt.h"

namespace mf {
namespace {

constexpr int kThr = 256;
#define MF_PPT_LENGTHS(X) X(16) X(32) X(64) X(96) X(128) X(192) X(256) X(384) X(512)
inline unsigned grid_of(size_t n) {
  size_t b = (n + kThr - 1) / kThr;
  if (b > 152u * 32u) b = 152u * 32u;
  return (unsigned)(b ? b : 1);
}

// signed index of get_k (grid_fft.hh:282-296): the Nyquist index stays positive
__device__ __forceinline__ int kidx(int i, int n) { return i - ((i > n / 2) ? n : 0); }

// z pass of a 3D complex transform: contiguous lines of L complex doubles
template <int L, bool INV, int LPB>
__global__ void __launch_bounds__(LPB * LineFFT<double, L, INV, 8, true>::TPL)
    k_zc2c(double2* __restrict__ data, int nlines, double scale, const double2* __restrict__ tw) {
  using F = LineFFT<double, L, INV, 8, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, ly = threadIdx.y;
  const int line = blockIdx.x * LPB + ly;
  const bool valid = line < nlines;
  double2* sm = reinterpret_cast<double2*>(smem_raw) + ly * padded_len(L, true);
  double2* p = data + (size_t)(valid ? line : 0) * L;
  double2 v[F::E];
#pragma unroll
  for (int s = 0; s < F::E; ++s) v[s] = valid ? p[F::in_index(t, s)] : make_double2(0.0, 0.0);
  F::run(v, t, sm, 1, tw, SyncBlock{});
  if (valid) {
#pragma unroll
    for (int s = 0; s < F::E; ++s) p[F::out_index(t, s)] = make_double2(v[s].x * scale, v[s].y * scale);
  }
}

template <int L, bool INV>
cudaError_t launch_zc2c(double2* data, int nlines, double scale, const double2* tw, cudaStream_t s) {
  using F = LineFFT<double, L, INV, 8, true>;
  constexpr int LPB = (F::TPL >= 256) ? 1 : 256 / F::TPL;
  const size_t smem = (size_t)LPB * padded_len(L, true) * sizeof(double2);
  auto kern = k_zc2c<L, INV, LPB>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<(nlines + LPB - 1) / LPB, dim3(F::TPL, LPB), smem, s>>>(data, nlines, scale, tw);
  return cudaGetLastError();
}

// growth-scaled k-space potential in FP64 on the padded real-transform layout
template <typename T>
__global__ void k_ppt_scale(const cplx<T>* __restrict__ src, double2* __restrict__ dst, size_t tot, double g) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const cplx<T> v = src[q];
    dst[q] = make_double2(g * (double)v.x, g * (double)v.y);
  }
}

__device__ __forceinline__ void atomic_max_pos(double* addr, double v) {
  // non-negative doubles order as their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// largest neighbour difference of phi (ic_generator.cc:703-719; the base
// index i stops at n-2 as in the reference)
__global__ void k_ppt_dphi_max(const double* __restrict__ phi, int n, double* maxd) {
  const size_t rs = (size_t)n + 2;
  const size_t tot = (size_t)(n - 1) * n * n;
  double m = 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < tot; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / ((size_t)n * n)), j = (int)((c / n) % n), k = (int)(c % n);
    const int jr = (j + 1) % n, kr = (k + 1) % n;
    const double pc = phi[((size_t)i * n + j) * rs + k];
    const double dx = fabs(phi[((size_t)(i + 1) * n + j) * rs + k] - pc);
    const double dy = fabs(phi[((size_t)i * n + jr) * rs + k] - pc);
    const double dz = fabs(phi[((size_t)i * n + j) * rs + kr] - pc);
    m = fmax(m, fmax(dx, fmax(dy, dz)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double red[kThr / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    atomic_max_pos(maxd, m);
  }
}

__device__ __forceinline__ double ppt_hbar(const double* maxd, double D) {
  return *maxd / M_PI / D * 1.01;  // hbar_safefac (ic_generator.cc:725-726)
}

// psi = sqrt(1 + C delta) exp(i (phi [+ phi2]) / hbar / D+) (ic_generator.cc:697-700, :729-738)
template <typename T>
__global__ void k_ppt_psi(double2* __restrict__ psi, const double* __restrict__ phi, const double* __restrict__ phi2,
                          const T* __restrict__ delta, double C, int n, double D, const double* maxd) {
  const size_t n3 = (size_t)n * n * n, rs = (size_t)n + 2;
  const double ih = 1.0 / ppt_hbar(maxd, D);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const size_t r = (c / n) * rs + c % n;
    const double ph = phi2 ? (phi[r] + phi2[r]) : phi[r];
    const double rho = delta ? sqrt(1.0 + C * (double)delta[r]) : sqrt(1.0 + C * 0.0);
    double sn, cs;
    sincos(ih * ph / D, &sn, &cs);
    psi[c] = make_double2(rho * cs, rho * sn);
  }
}

// one drift step psi_k exp(-i hbar k^2 D+ / 2) (ic_generator.cc:743-748)
__global__ void k_ppt_drift(double2* __restrict__ psi, int n, double kfac, double D, const double* maxd) {
  const size_t n3 = (size_t)n * n * n;
  const double hb = ppt_hbar(maxd, D);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / ((size_t)n * n)), j = (int)((c / n) % n), k = (int)(c % n);
    const double kx = kidx(i, n) * kfac, ky = kidx(j, n) * kfac, kz = kidx(k, n) * kfac;
    const double a = -0.5 * hb * (kx * kx + ky * ky + kz * kz) * D;
    double sn, cs;
    sincos(a, &sn, &cs);
    const double2 v = psi[c];
    psi[c] = make_double2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
  }
}

// psi exp(i phi2 / hbar / D+) after the drift (ic_generator.cc:751-755)
__global__ void k_ppt_kick2(double2* __restrict__ psi, const double* __restrict__ phi2, int n, double D,
                            const double* maxd) {
  const size_t n3 = (size_t)n * n * n, rs = (size_t)n + 2;
  const double ih = 1.0 / ppt_hbar(maxd, D);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    double sn, cs;
    sincos(ih * phi2[(c / n) * rs + c % n] / D, &sn, &cs);
    const double2 v = psi[c];
    psi[c] = make_double2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
  }
}

// rho = |psi|^2 - 1 (ic_generator.cc:760-763)
__global__ void k_ppt_rho(const double2* __restrict__ psi, double* __restrict__ rho, size_t n3) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const double2 v = psi[c];
    rho[c] = v.x * v.x + v.y * v.y - 1.0;
  }
}

// grad_psi_k = psi_k i k_d (ic_generator.cc:778-780)
__global__ void k_ppt_grad(const double2* __restrict__ psik, double2* __restrict__ g, int n, double kfac, int d) {
  const size_t n3 = (size_t)n * n * n;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / ((size_t)n * n)), j = (int)((c / n) % n), k = (int)(c % n);
    const double kd = (d == 0 ? kidx(i, n) : (d == 1 ? kidx(j, n) : kidx(k, n))) * kfac;
    const double2 v = psik[c];
    g[c] = make_double2(-kd * v.y, kd * v.x);
  }
}

// v_d = vunit Re((conj(psi) grad - psi conj(grad)) / (2i / hbar)) / (1 + rho)
// (ic_generator.cc:783-786)
__global__ void k_ppt_vel(const double2* __restrict__ psi, const double2* __restrict__ g,
                          const double* __restrict__ rho, double* __restrict__ v, size_t n3, double vunit, double D,
                          const double* maxd) {
  const double hb = ppt_hbar(maxd, D);
  const double den = 2.0 / hb;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const double2 p = psi[c], q = g[c];
    // conj(p) q - p conj(q) = 2 i Im(conj(p) q); divided by (0, 2/hbar): real part Im(conj(p) q) 2 / (2/hbar)
    const double im = p.x * q.y - p.y * q.x;
    v[c] = vunit * ((2.0 * im) / den) / (1.0 + rho[c]);
  }
}

}  // namespace

cudaError_t fft3d_c2c_f64(mf_ctx* c, double2* data, int n, bool inverse) {
  cudaStream_t s = c->stream;
  const double2* tw = c->tw.get<double>(n, s);
  if (!tw) return cudaErrorMemoryAllocation;
  const double scale = 1.0 / std::sqrt((double)n * (double)n * (double)n);
  cudaError_t e = cudaErrorInvalidValue;
  {
    LaunchScope ls(c, KK_FFT_Z);
#define CASE(LL)                                                                                    \
  case LL:                                                                                          \
    e = inverse ? launch_zc2c<LL, true>(data, n * n, scale, tw, s) : launch_zc2c<LL, false>(data, n * n, scale, tw, s); \
    break;
    switch (n) { MF_PPT_LENGTHS(CASE) default: break; }
#undef CASE
  }
  if (e != cudaSuccess) return e;
  {
    LaunchScope ls(c, KK_FFT_COL);
    e = Launch<double>::colfft_plain(n, inverse, PlainStridedOp<double>{data, n, (long long)n * n, 1.0}, n, n, tw, s);
  }
  if (e != cudaSuccess) return e;
  LaunchScope ls(c, KK_FFT_COL);
  return Launch<double>::colfft_plain(n, inverse, PlainStridedOp<double>{data, (long long)n * n, n, 1.0}, n, n, tw, s);
}

template <typename T>
cudaError_t ppt_eulerian(mf_ctx* c, const PPTArgs& a) {
  cudaStream_t s = c->stream;
  const int n = a.n;
  const size_t n3 = (size_t)n * n * n, nk = (size_t)n * n * (n / 2 + 1);
  const double kfac = 2.0 * M_PI / a.L;
  cudaError_t e;
#define CK(x)                          \
  do {                                 \
    e = (x);                           \
    if (e != cudaSuccess) return e;    \
  } while (0)
  // real-space phi and phi2 (growth-scaled, as after ic_generator.cc:550-563)
  {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_scale<T><<<grid_of(nk), kThr, 0, s>>>((const cplx<T>*)a.f0, (double2*)a.phi_r, nk, a.g1);
    CK(cudaGetLastError());
  }
  CK(fft3d_c2r<double>(c, a.phi_r, n));
  if (a.f1) {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_scale<T><<<grid_of(nk), kThr, 0, s>>>((const cplx<T>*)a.f1, (double2*)a.phi2_r, nk, a.g2);
    CK(cudaGetLastError());
  }
  if (a.f1) CK(fft3d_c2r<double>(c, a.phi2_r, n));
  // the species' delta_bc in real space (no relative-velocity amplitude)
  if (a.delta_k) {
    CK(cudaMemcpyAsync(a.delta_r, a.delta_k, grid_reals(n) * sizeof(T), cudaMemcpyDeviceToDevice, s));
    CK(fft3d_c2r<T>(c, (T*)a.delta_r, n));
  }
  CK(cudaMemsetAsync(a.maxd, 0, sizeof(double), s));
  {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_dphi_max<<<grid_of((size_t)(n - 1) * n * n), kThr, 0, s>>>(a.phi_r, n, a.maxd);
    CK(cudaGetLastError());
  }
  {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_psi<T><<<grid_of(n3), kThr, 0, s>>>(a.psi, a.phi_r, a.f1 ? a.phi2_r : nullptr,
                                               a.delta_k ? (const T*)a.delta_r : nullptr, a.C, n, a.D, a.maxd);
    CK(cudaGetLastError());
  }
  CK(fft3d_c2c_f64(c, a.psi, n, false));
  {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_drift<<<grid_of(n3), kThr, 0, s>>>(a.psi, n, kfac, a.D, a.maxd);
    CK(cudaGetLastError());
  }
  CK(fft3d_c2c_f64(c, a.psi, n, true));
  if (a.f1) {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_kick2<<<grid_of(n3), kThr, 0, s>>>(a.psi, a.phi2_r, n, a.D, a.maxd);
    CK(cudaGetLastError());
  }
  {
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_rho<<<grid_of(n3), kThr, 0, s>>>(a.psi, a.rho_out, n3);
    CK(cudaGetLastError());
  }
  // velocities: psi to k-space once, then per component i k_d psi_k back to real space
  CK(cudaMemcpyAsync(a.grad, a.psi, n3 * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  CK(fft3d_c2c_f64(c, a.grad, n, false));
  double2* psik = a.grad;
  double2* g = a.grad + n3;
  for (int d = 0; d < 3; ++d) {
    {
      LaunchScope ls(c, KK_POINTWISE);
      k_ppt_grad<<<grid_of(n3), kThr, 0, s>>>(psik, g, n, kfac, d);
      CK(cudaGetLastError());
    }
    CK(fft3d_c2c_f64(c, g, n, true));
    LaunchScope ls(c, KK_POINTWISE);
    k_ppt_vel<<<grid_of(n3), kThr, 0, s>>>(a.psi, g, a.rho_out, a.vel_out + (size_t)d * n3, n3, a.vunit, a.D, a.maxd);
    CK(cudaGetLastError());
  }
#undef CK
  return cudaSuccess;
}

template cudaError_t ppt_eulerian<float>(mf_ctx*, const PPTArgs&);
template cudaError_t ppt_eulerian<double>(mf_ctx*, const PPTArgs&);

}  // namespace mf

extern "C" int mf_cgrid_fft(mf_ctx* c, void* data, int n, int inverse) {
  if (!c || !data) return MF_ERR_ARG;
  if (!mf::grid_size_supported(n)) return mf::set_err(c, MF_ERR_SHAPE, "mf_cgrid_fft: unsupported grid size");
  cudaSetDevice(c->device);
  const cudaError_t e = mf::fft3d_c2c_f64(c, static_cast<double2*>(data), n, inverse != 0);
  return e == cudaSuccess ? MF_OK : mf::cuda_err(c, e, "mf_cgrid_fft");
}
