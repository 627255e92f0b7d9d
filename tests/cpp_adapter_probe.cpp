// Exercises the C++ adapter (include/monofonic_gb300.hpp) the way
// ic_generator.cc uses the reference API.  Linked against the host fake of
// the C ABI (tests/cpp_adapter_fake.cpp) it checks what the adapter passes
// to the library; linked against libmfgpu.so on a GPU it runs the same calls
// on the device.  Prints "ok" and exits 0 when every check holds.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>

#include "monofonic_gb300.hpp"

using mfgpu::Grid_FFT;
using mfgpu::OrszagConvolver;
namespace op = mfgpu::op;

#define CHECK(c)                                                 \
  do {                                                           \
    if (!(c)) {                                                  \
      std::printf("check failed at line %d: %s\n", __LINE__, #c); \
      return 1;                                                  \
    }                                                            \
  } while (0)

#ifdef MF_FAKE_ABI
extern "C" {
extern mf_operand fake_last_opnd[3];
extern int fake_last_nopnd, fake_last_op, fake_last_invlap;
extern double fake_last_x;
extern mf_grid* fake_last_out;
}
#endif

template <typename real_t>
int run(mfgpu::context& ctx) {
  const size_t n = 16;
  const real_t L = 100;
  Grid_FFT<real_t> phi(ctx, {n, n, n}, {L, L, L});
  Grid_FFT<real_t> phi2(ctx, {n, n, n}, {L, L, L}, false);  // not allocated until needed
  CHECK(phi.is_allocated() && !phi2.is_allocated());
  phi2.allocate();
  CHECK(phi.space() == mfgpu::rspace_id && phi.size(3) == n + 2 && phi.get_idx(1, 2, 3) == (1 * n + 2) * (n + 2) + 3);

  // a known real field through Fill_Grid, then single-element reads
  std::vector<double> x(n * n * n);
  for (size_t i = 0; i < x.size(); ++i) x[i] = std::sin(0.37 * double(i)) + 0.01 * double(i % 7);
  phi.fill_real64(x);
  CHECK(phi.relem(2, 3, 4) == real_t(x[(2 * n + 3) * n + 4]));
  std::vector<real_t> padded;
  phi.download(padded);
  CHECK(padded.size() == (n + 2) * n * n && padded[phi.get_idx(5, 6, 7)] == real_t(x[(5 * n + 6) * n + 7]));

  // functors on the host mirror, as ic_generator.cc:341-457 uses them
  {
    Grid_FFT<real_t> a(ctx, {n, n, n}, {L, L, L}), b(ctx, {n, n, n}, {L, L, L});
    a.fill_real64(x);
    const real_t a234 = a.relem(2, 3, 4);
    a.apply_function_r_dep([](auto v, auto r) { return v + r.z; });
    CHECK(a.relem(2, 3, 4) == a234 + real_t(4) * a.get_dx(2));
    b.assign_function_of_grids_r([](auto u, auto w) { return u - w; }, a, a);
    CHECK(b.relem(2, 3, 4) == real_t(0) && b.space() == mfgpu::rspace_id);
    a.apply_function_r([](auto v) { return v * real_t(2); });
    CHECK(a.relem(2, 3, 4) == (a234 + real_t(4) * a.get_dx(2)) * real_t(2));
    a.FourierTransformForward();
    const std::complex<real_t> c = a.kelem(1, 2, 3);
    const auto k = a.template get_k<real_t>(1, 2, 3);
    a.apply_function_k_dep([](auto v, auto kv) { return v * kv.norm_squared(); });
    const std::complex<real_t> c2 = c * k.norm_squared();
    CHECK(a.kelem(1, 2, 3) == c2 && a.space() == mfgpu::kspace_id);
    b.assign_function_of_grids_kdep([](auto kv, auto u, auto w) { return u * w * kv.x; }, a, a);
    CHECK(b.kelem(1, 2, 3) == c2 * c2 * k.x);
    b.assign_function_of_grids_ijk([](auto ijk, auto u) { return u * real_t(ijk[0] + ijk[2]); }, a);
    CHECK(b.kelem(1, 2, 3) == c2 * real_t(4));
    b.assign_function_of_grids_k([](auto u) { return u + u; }, a);
    b.apply_function_k([](auto v) { return std::conj(v); });
    CHECK(b.kelem(1, 2, 3) == std::conj(c2 + c2));
  }

  phi.FourierTransformForward();
  CHECK(phi.space() == mfgpu::kspace_id && phi.size(2) == n / 2 + 1 && phi.size(3) == n / 2 + 1);
  const std::complex<real_t> k123 = phi.kelem(1, 2, 3);
  phi.download(padded);
  CHECK(k123 == std::complex<real_t>(padded[2 * phi.get_idx(1, 2, 3)], padded[2 * phi.get_idx(1, 2, 3) + 1]));
  bool threw = false;
  try {
    (void)phi.kelem(n, 0, 0);
  } catch (const std::out_of_range&) {
    threw = true;
  }
  CHECK(threw);

  // wave vectors, gradients and the Laplacian of grid_fft.hh:281-390
  const real_t kf = real_t(2.0 * M_PI / double(L));
  const auto kk = phi.template get_k<real_t>(9, 3, 8);
  CHECK(kk[0] == real_t(-7) * kf && kk[1] == real_t(3) * kf && kk[2] == real_t(8) * kf);
  CHECK(phi.gradient(2, {1, 1, n / 2}) == std::complex<real_t>(0, 0));
  CHECK(phi.gradient(0, {9, 1, 1}) == std::complex<real_t>(0, real_t(-7) * kf));
  CHECK(phi.laplacian({9, 3, 8}) == -(kk[0] * kk[0] + kk[1] * kk[1] + kk[2] * kk[2]));

  // the source terms of phi(2) as ic_generator.cc:471-488 writes them
  OrszagConvolver<real_t> Conv(ctx, {n, n, n}, {L, L, L});
  phi2.FourierTransformForward(false);
  Conv.convolve_SumOfHessians(phi, {0, 0}, phi, {1, 1}, {2, 2}, op::assign_to(phi2));
#ifdef MF_FAKE_ABI
  CHECK(fake_last_nopnd == 2 && fake_last_op == MF_OP_ASSIGN && fake_last_out == phi2.handle());
  CHECK(fake_last_opnd[0].kind == MF_OPND_HESS && fake_last_opnd[0].d[0] == 0 && fake_last_opnd[0].d[1] == 0);
  CHECK(fake_last_opnd[1].kind == MF_OPND_SUM && fake_last_opnd[1].d[0] == 1 && fake_last_opnd[1].d[1] == 1 &&
        fake_last_opnd[1].d[2] == 2 && fake_last_opnd[1].d[3] == 2);
#endif
  Conv.convolve_Hessians(phi, {1, 1}, phi, {2, 2}, op::add_to(phi2));
  Conv.convolve_Hessians(phi, {0, 1}, phi, {0, 1}, op::subtract_from(phi2));
  Conv.convolve_DifferenceOfHessians(phi, {0, 1}, phi, {0, 2}, {1, 2}, op::multiply_add_to(phi2, 2.5));
#ifdef MF_FAKE_ABI
  CHECK(fake_last_op == MF_OP_AXPY && fake_last_x == 2.5 && fake_last_opnd[1].kind == MF_OPND_DIFF);
  CHECK(fake_last_opnd[1].d[0] == 0 && fake_last_opnd[1].d[1] == 2 && fake_last_opnd[1].d[2] == 1 &&
        fake_last_opnd[1].d[3] == 2);
#endif
  Conv.convolve_Gradients(phi, {0}, phi, {2}, op::add_to(phi2));
#ifdef MF_FAKE_ABI
  CHECK(fake_last_op == MF_OP_ADD && fake_last_opnd[0].kind == MF_OPND_GRAD && fake_last_opnd[1].d[0] == 2);
#endif
  Conv.convolve_Hessians(phi, {0, 0}, phi, {1, 1}, phi, {2, 2}, op::assign_to(phi2));
#ifdef MF_FAKE_ABI
  CHECK(fake_last_nopnd == 3 && fake_last_opnd[2].kind == MF_OPND_HESS && fake_last_opnd[2].d[0] == 2);
#endif
  Conv.convolve_Hessians_then_InverseLaplacian(phi, {1, 2}, phi, {1, 2}, op::subtract_from(phi2));
#ifdef MF_FAKE_ABI
  CHECK(fake_last_invlap == 1 && fake_last_op == MF_OP_SUB);
#endif
  phi2.apply_InverseLaplacian();
  phi2.zero_DC_mode();
  phi2 *= real_t(-3.0 / 7.0);
  phi2.shift_field({real_t(0.5), real_t(0.25), real_t(0)}, false);

  std::vector<double> bk, bP, beP;
  std::vector<size_t> cnt;
  phi.Compute_PowerSpectrum(bk, bP, beP, cnt);
  CHECK(bk.size() == bP.size() && bP.size() == cnt.size() && !bk.empty());

  // failures surface as mfgpu::error with the library's status
  threw = false;
  try {
    Grid_FFT<real_t> bad(ctx, {100, 100, 100}, {L, L, L});
  } catch (const mfgpu::error& e) {
    threw = e.code() == MF_ERR_SHAPE && std::strstr(e.what(), "mf_grid_create") != nullptr;
  }
  CHECK(threw);
  threw = false;
  try {
    Grid_FFT<real_t> unalloc(ctx, {n, n, n}, {L, L, L}, false);
    unalloc.zero();
  } catch (const mfgpu::error& e) {
    threw = e.code() == MF_ERR_STATE;
  }
  CHECK(threw);
  phi.FourierTransformBackward();
  CHECK(phi.space() == mfgpu::rspace_id);
  return 0;
}

int main() {
  try {
    mfgpu::context ctx(0);
    if (run<double>(ctx) || run<float>(ctx)) return 1;
  } catch (const std::exception& e) {
    std::printf("exception: %s\n", e.what());
    return 2;
  }
  std::printf("ok\n");
  return 0;
}
