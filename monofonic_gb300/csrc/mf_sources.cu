// Real-space products of the LPT source terms (ic_generator.cc:471-545) over
// the shared padded real fields, as streaming kernels with the formulas fixed
// at compile time: every field is read once per pass and several targets'
// product sums are written in the same pass.
//
// Field numbering: 0..5 Hessians of phi (00, 11, 22, 01, 02, 12), 6..11 the
// same Hessians of phi(2), 12..16 the truncated convolve3 pair products.
#include <cstddef>
#include <type_traits>
#include <utility>

#include "mf_runtime.h"

namespace mf {

struct SrcTerm {
  int out, a, b;
  double w;
};

// Hessian field of directions (a, b)
constexpr int src_hx(int a, int b) {
  return (a > b) ? src_hx(b, a) : ((a == b) ? a : (a == 0 ? (b == 1 ? 3 : 4) : 5));
}
constexpr int src_dp(int d) { return (d + 1) % 3; }
constexpr int src_dpp(int d) { return (d + 2) % 3; }

// nabla^2 phi(2) = phi,00 (phi,11 + phi,22) + phi,11 phi,22 - phi,01^2 - phi,02^2 - phi,12^2
struct SrcSetPhi2 {
  static constexpr SrcTerm terms[] = {{0, 0, 1, 1.0}, {0, 0, 2, 1.0}, {0, 1, 2, 1.0},
                                      {0, 3, 3, -1.0}, {0, 4, 4, -1.0}, {0, 5, 5, -1.0}};
};
// first stages of the five convolve3 terms: phi,00 phi,11 / phi,01 phi,02 /
// phi,12^2 / phi,02^2 / phi,01^2
struct SrcSetPairs {
  static constexpr SrcTerm terms[] = {{0, 0, 1, 1.0}, {1, 3, 4, 1.0}, {2, 5, 5, 1.0}, {3, 4, 4, 1.0}, {4, 3, 3, 1.0}};
};
// the phi(2) source (output 0) and the five convolve3 pairs (outputs 1..5):
// both read only the Hessians of phi, so one pass serves a 3LPT run
struct SrcSetPhi2Pairs {
  static constexpr SrcTerm terms[] = {{0, 0, 1, 1.0},  {0, 0, 2, 1.0},  {0, 1, 2, 1.0},  {0, 3, 3, -1.0},
                                      {0, 4, 4, -1.0}, {0, 5, 5, -1.0}, {1, 0, 1, 1.0},  {2, 3, 4, 1.0},
                                      {3, 5, 5, 1.0},  {4, 4, 4, 1.0},  {5, 3, 3, 1.0}};
};
// phi(3) (output 0) and A(3) x, y, z (outputs 1..3)
#define MF_A3_TERMS(d)                                                                                       \
  {1 + d, 6 + src_hx(d, src_dp(d)), src_hx(d, src_dpp(d)), 1.0},                                             \
      {1 + d, 6 + src_hx(d, src_dpp(d)), src_hx(d, src_dp(d)), -1.0},                                        \
      {1 + d, src_hx(src_dp(d), src_dpp(d)), 6 + src_hx(src_dp(d), src_dp(d)), 1.0},                        \
      {1 + d, src_hx(src_dp(d), src_dpp(d)), 6 + src_hx(src_dpp(d), src_dpp(d)), -1.0},                     \
      {1 + d, 6 + src_hx(src_dp(d), src_dpp(d)), src_hx(src_dp(d), src_dp(d)), -1.0},                       \
      {1 + d, 6 + src_hx(src_dp(d), src_dpp(d)), src_hx(src_dpp(d), src_dpp(d)), 1.0}
struct SrcSetPhi3A3 {
  static constexpr double a5 = -5.0 / 7.0, a10 = 10.0 / 7.0;
  static constexpr SrcTerm terms[] = {
      {0, 12, 2, 1.0}, {0, 13, 5, 2.0}, {0, 14, 0, -1.0}, {0, 15, 1, -1.0}, {0, 16, 2, -1.0},
      {0, 0, 7, a5},   {0, 0, 8, a5},   {0, 1, 8, a5},    {0, 1, 6, a5},    {0, 2, 6, a5},
      {0, 2, 7, a5},   {0, 3, 9, a10},  {0, 4, 10, a10},  {0, 5, 11, a10},
      MF_A3_TERMS(0),  MF_A3_TERMS(1),  MF_A3_TERMS(2)};
};
#undef MF_A3_TERMS

template <class SET>
constexpr size_t src_nterm() { return sizeof(SET::terms) / sizeof(SrcTerm); }
template <class SET>
constexpr bool src_uses(int f) {
  for (size_t t = 0; t < src_nterm<SET>(); ++t)
    if (SET::terms[t].a == f || SET::terms[t].b == f) return true;
  return false;
}
template <class SET>
constexpr int src_nout() {
  int n = 0;
  for (size_t t = 0; t < src_nterm<SET>(); ++t)
    if (SET::terms[t].out + 1 > n) n = SET::terms[t].out + 1;
  return n;
}

template <typename T>
struct SrcPtrs {
  const T* f[kSrcFields];
  T* out[kSrcOutputs];
};

template <class SET>
constexpr unsigned src_mask() {
  unsigned m = 0;
  for (int f = 0; f < kSrcFields; ++f)
    if (src_uses<SET>(f)) m |= 1u << f;
  return m;
}

// one term, its indices and weight fixed at compile time
template <typename T, class SET, size_t I>
__device__ __forceinline__ void src_term(const T (&fv)[kSrcFields][16 / sizeof(T)],
                                         T (&acc)[kSrcOutputs][16 / sizeof(T)]) {
  constexpr SrcTerm tm = SET::terms[I];
  constexpr T w = T(tm.w);
#pragma unroll
  for (int j = 0; j < (int)(16 / sizeof(T)); ++j) acc[tm.out][j] += w * (fv[tm.a][j] * fv[tm.b][j]);
}

template <typename T, class SET, size_t... I>
__device__ __forceinline__ void src_accumulate(const T (&fv)[kSrcFields][16 / sizeof(T)],
                                               T (&acc)[kSrcOutputs][16 / sizeof(T)], std::index_sequence<I...>) {
  (src_term<T, SET, I>(fv, acc), ...);
}

template <typename T, class SET>
__global__ void __launch_bounds__(256) k_sources(SrcPtrs<T> p, size_t nvec) {
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  constexpr int W = 16 / sizeof(T);
  constexpr int NO = src_nout<SET>();
  constexpr unsigned MASK = src_mask<SET>();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nvec; i += (size_t)gridDim.x * blockDim.x) {
    T fv[kSrcFields][W];
#pragma unroll
    for (int f = 0; f < kSrcFields; ++f) {
      if (MASK & (1u << f)) {
        const V v = reinterpret_cast<const V*>(p.f[f])[i];
        const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
        for (int j = 0; j < W; ++j) fv[f][j] = e[j];
      }
    }
    T acc[kSrcOutputs][W] = {};
    src_accumulate<T, SET>(fv, acc, std::make_index_sequence<src_nterm<SET>()>{});
#pragma unroll
    for (int o = 0; o < NO; ++o) {
      V r;
      T* re = reinterpret_cast<T*>(&r);
#pragma unroll
      for (int j = 0; j < W; ++j) re[j] = acc[o][j];
      reinterpret_cast<V*>(p.out[o])[i] = r;
    }
  }
}

namespace {

template <typename T, class SET>
cudaError_t launch_sources(const T* const* fields, T* const* outs, size_t n, cudaStream_t s) {
  constexpr size_t W = 16 / sizeof(T);
  if (n % W) return cudaErrorInvalidValue;
  SrcPtrs<T> p{};
  for (int f = 0; f < kSrcFields; ++f) p.f[f] = fields[f];
  for (int o = 0; o < src_nout<SET>(); ++o) {
    if (!outs[o]) return cudaErrorInvalidValue;
    p.out[o] = outs[o];
  }
  for (int f = 0; f < kSrcFields; ++f)
    if (src_uses<SET>(f) && !fields[f]) return cudaErrorInvalidValue;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t nvec = n / W;
  size_t grid = (nvec + 255) / 256;
  const size_t cap = (size_t)nsm * 8;
  if (grid > cap) grid = cap;
  k_sources<T, SET><<<(unsigned)(grid ? grid : 1), 256, 0, s>>>(p, nvec);
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t pw_sources(int set, const T* const* fields, T* const* outs, size_t n, cudaStream_t s) {
  switch (set) {
    case SRC_PHI2: return launch_sources<T, SrcSetPhi2>(fields, outs, n, s);
    case SRC_PAIRS: return launch_sources<T, SrcSetPairs>(fields, outs, n, s);
    case SRC_PHI3_A3: return launch_sources<T, SrcSetPhi3A3>(fields, outs, n, s);
    case SRC_PHI2_PAIRS: return launch_sources<T, SrcSetPhi2Pairs>(fields, outs, n, s);
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t pw_sources<float>(int, const float* const*, float* const*, size_t, cudaStream_t);
template cudaError_t pw_sources<double>(int, const double* const*, double* const*, size_t, cudaStream_t);

}  // namespace mf
