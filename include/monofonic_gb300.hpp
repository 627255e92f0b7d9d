/*
 * monofonic_gb300.hpp -- C++ mirror of monofonIC's field / convolver /
 * operator API over the C ABI of libmfgpu (header only).
 *
 *   mfgpu::Grid_FFT<real_t>         include/grid_fft.hh:40-914
 *   mfgpu::OrszagConvolver<real_t>  include/convolution.hh:429-669
 *   mfgpu::NaiveConvolver<real_t>   include/convolution.hh:296-426
 *   mfgpu::op::assign_to ...        include/operators.hh:25-35
 *
 * The names, argument order and defaults are the reference's, so code
 * written against them compiles with `using mfgpu::Grid_FFT;` (and the like)
 * in place of the reference headers: `Grid_FFT<real_t> phi({n, n, n}, {L, L,
 * L});` allocates the field in HBM, `Conv.convolve_Hessians(phi, {0, 1}, phi,
 * {2, 2}, op::add_to(phi2));` runs the convolution on the GPU.  real_t is
 * double (plain FP64) or float (the FP32-bulk form).  The grids live on one
 * device; the MPI slab decomposition of the reference has no counterpart.
 *
 * Differences that follow from the data living in HBM:
 * - relem / kelem read one element back to the host (after the context's
 *   stream drains); move whole fields with upload / download instead;
 * - op:: output operators name the target grid and the operation instead of
 *   being host lambdas; the convolver applies them in its last store;
 * - failures throw mfgpu::error (a std::runtime_error, as the reference
 *   throws) carrying the library's status code and message.
 */
#ifndef MONOFONIC_GB300_HPP
#define MONOFONIC_GB300_HPP

#include <array>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "monofonic_gb300.h"

namespace mfgpu {

/* a failed library call: the status code (MF_ERR_*) and its message */
class error : public std::runtime_error {
 public:
  error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

namespace detail {
inline void check(const mf_ctx* c, int rc, const char* what) {
  if (rc != MF_OK) throw error(rc, std::string(what) + ": " + (c ? mf_last_error(c) : "failed"));
}
template <typename T>
struct prec_of;
template <>
struct prec_of<double> {
  static constexpr int value = MF_PREC_F64;
};
template <>
struct prec_of<float> {
  static constexpr int value = MF_PREC_F32;
};
constexpr double two_pi = 6.283185307179586476925286766559;
}  // namespace detail

/* the device and stream the grids and convolvers work on; replaces the
 * FFTW / OpenMP set-up of src/main.cc:150-181 */
class context {
 public:
  explicit context(int device = 0) { detail::check(nullptr, mf_ctx_create(device, &c_), "mf_ctx_create"); }
  ~context() {
    if (c_) mf_ctx_destroy(c_);
  }
  context(const context&) = delete;
  context& operator=(const context&) = delete;
  mf_ctx* get() const noexcept { return c_; }
  void synchronize() const { detail::check(c_, mf_ctx_synchronize(c_), "mf_ctx_synchronize"); }

 private:
  mf_ctx* c_ = nullptr;
};

/* the context of objects constructed without one: device 0, created on
 * first use */
inline context& default_context() {
  static context ctx(0);
  return ctx;
}

/* include/grid_fft.hh:29 */
enum space_t { kspace_id, rspace_id };

/* the 3-vector the reference's functors receive (include/math/vec3.hh:23-110:
 * x, y, z, operator[], dot, norm_squared, norm) */
template <typename T>
struct vec3 {
  T x{}, y{}, z{};
  T& operator[](size_t i) noexcept { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](size_t i) const noexcept { return i == 0 ? x : (i == 1 ? y : z); }
  T dot(const vec3& a) const noexcept { return x * a.x + y * a.y + z * a.z; }
  T norm_squared() const noexcept { return dot(*this); }
  T norm() const noexcept { return std::sqrt(norm_squared()); }
};

/* Grid_FFT<real_t>: an n^3 field in HBM in the reference's in-place padded
 * layout, (n+2) reals per row in real space, n/2+1 complex per row in
 * k-space (grid_fft.hh:184-216) */
template <typename data_t>
class Grid_FFT {
  static_assert(std::is_same<data_t, double>::value || std::is_same<data_t, float>::value,
                "Grid_FFT<real_t>: real_t is double or float");

 public:
  using real_t = data_t;
  using ccomplex_t = std::complex<real_t>;

  /* grid_fft.hh:77-84 */
  Grid_FFT(const std::array<size_t, 3>& N, const std::array<real_t, 3>& L, bool allocate = true,
           space_t initialspace = rspace_id)
      : Grid_FFT(default_context(), N, L, allocate, initialspace) {}
  Grid_FFT(context& ctx, const std::array<size_t, 3>& N, const std::array<real_t, 3>& L, bool allocate = true,
           space_t initialspace = rspace_id)
      : ctx_(&ctx), n_(N), length_(L), space0_(initialspace) {
    if (N[0] != N[1] || N[1] != N[2] || L[0] != L[1] || L[1] != L[2])
      throw error(MF_ERR_SHAPE, "Grid_FFT: cubic grids and boxes only");
    if (allocate) this->allocate();
  }
  ~Grid_FFT() { reset(); }
  Grid_FFT(const Grid_FFT&) = delete;
  Grid_FFT& operator=(const Grid_FFT&) = delete;

  /* src/grid_fft.cc:40-112 and grid_fft.hh:95-109 */
  void allocate() {
    if (!g_)
      detail::check(ctx_->get(),
                    mf_grid_create(ctx_->get(), static_cast<int>(n_[0]), static_cast<double>(length_[0]),
                                   detail::prec_of<real_t>::value, space0_ == kspace_id ? MF_SPACE_K : MF_SPACE_R,
                                   &g_),
                    "mf_grid_create");
  }
  void reset() {
    if (g_) mf_grid_destroy(g_);
    g_ = nullptr;
  }
  bool is_allocated() const noexcept { return g_ != nullptr; }
  mf_grid* handle() const {
    if (!g_) throw error(MF_ERR_STATE, "Grid_FFT: the grid is not allocated");
    return g_;
  }
  context& get_context() const noexcept { return *ctx_; }

  space_t space() const {
    int s = MF_SPACE_R;
    detail::check(ctx_->get(), mf_grid_info(handle(), nullptr, nullptr, &s, nullptr, nullptr), "mf_grid_info");
    return s == MF_SPACE_K ? kspace_id : rspace_id;
  }

  /* sizes_ of src/grid_fft.cc:100-110: extents and the stored row length */
  size_t size(size_t i) const {
    const size_t n = n_[0];
    const bool k = space() == kspace_id;
    const size_t s[4] = {n, n, k ? n / 2 + 1 : n, k ? n / 2 + 1 : n + 2};
    return s[i];
  }
  size_t get_idx(size_t i, size_t j, size_t k) const { return (i * size(1) + j) * size(3) + k; }
  real_t get_dx(int idim) const { return length_[idim] / static_cast<real_t>(n_[idim]); }
  std::array<size_t, 3> get_k3(size_t i, size_t j, size_t k) const { return {i, j, k}; }

  /* grid_fft.hh:218-228 */
  template <typename ft>
  vec3<ft> get_r(size_t i, size_t j, size_t k) const {
    vec3<ft> r;
    r.x = static_cast<ft>(static_cast<real_t>(i) * get_dx(0));
    r.y = static_cast<ft>(static_cast<real_t>(j) * get_dx(1));
    r.z = static_cast<ft>(static_cast<real_t>(k) * get_dx(2));
    return r;
  }
  /* grid_fft.hh:281-296: (idx - n [idx > n/2]) 2pi/L per axis */
  template <typename ft>
  vec3<ft> get_k(size_t i, size_t j, size_t k) const {
    const size_t idx[3] = {i, j, k};
    vec3<ft> kk;
    for (int d = 0; d < 3; ++d) {
      const real_t kfac = static_cast<real_t>(detail::two_pi / length_[d]);
      kk[d] = static_cast<ft>((static_cast<real_t>(idx[d]) -
                               static_cast<real_t>(idx[d] > n_[d] / 2) * static_cast<real_t>(n_[d])) *
                              kfac);
    }
    return kk;
  }
  /* grid_fft.hh:376-385: i k_idim, zero at that axis' Nyquist index */
  ccomplex_t gradient(const int idim, std::array<size_t, 3> ijk) const {
    if (ijk[idim] == n_[idim] / 2) return ccomplex_t(0, 0);
    return ccomplex_t(0, get_k<real_t>(ijk[0], ijk[1], ijk[2])[idim]);
  }
  /* grid_fft.hh:387-390 */
  real_t laplacian(const std::array<size_t, 3>& ijk) const {
    const auto kk = get_k<real_t>(ijk[0], ijk[1], ijk[2]);
    return -(kk[0] * kk[0] + kk[1] * kk[1] + kk[2] * kk[2]);
  }

  /* src/grid_fft.cc:208-270 */
  void FourierTransformForward(bool do_transform = true) {
    detail::check(ctx_->get(), mf_grid_fft_forward(handle(), do_transform ? 1 : 0), "FourierTransformForward");
  }
  void FourierTransformBackward(bool do_transform = true) {
    detail::check(ctx_->get(), mf_grid_fft_backward(handle(), do_transform ? 1 : 0), "FourierTransformBackward");
  }
  void zero() { detail::check(ctx_->get(), mf_grid_zero(handle()), "zero"); }
  void zero_DC_mode() { detail::check(ctx_->get(), mf_grid_zero_dc(handle()), "zero_DC_mode"); }
  void apply_InverseLaplacian() {
    detail::check(ctx_->get(), mf_grid_inverse_laplacian(handle()), "apply_InverseLaplacian");
  }
  Grid_FFT& operator*=(data_t x) {
    detail::check(ctx_->get(), mf_grid_scale(handle(), static_cast<double>(x)), "operator*=");
    return *this;
  }
  /* grid_fft.hh:832-842, s in units of the cell size */
  void shift_field(const std::array<real_t, 3>& s, bool transform_back = true) {
    const double sd[3] = {static_cast<double>(s[0]), static_cast<double>(s[1]), static_cast<double>(s[2])};
    detail::check(ctx_->get(), mf_grid_shift(handle(), sd, transform_back ? 1 : 0), "shift_field");
  }
  /* src/grid_fft.cc:1133-1210 */
  void Compute_PowerSpectrum(std::vector<double>& bin_k, std::vector<double>& bin_P, std::vector<double>& bin_eP,
                             std::vector<size_t>& bin_count) {
    const int cap = static_cast<int>(n_[0]);
    std::vector<int64_t> cnt(cap);
    bin_k.assign(cap, 0.0);
    bin_P.assign(cap, 0.0);
    bin_eP.assign(cap, 0.0);
    int nb = 0;
    detail::check(ctx_->get(),
                  mf_grid_power_spectrum(handle(), bin_k.data(), bin_P.data(), bin_eP.data(), cnt.data(), cap, &nb),
                  "Compute_PowerSpectrum");
    bin_k.resize(nb);
    bin_P.resize(nb);
    bin_eP.resize(nb);
    bin_count.assign(cnt.begin(), cnt.begin() + nb);
  }
  /* src/grid_fft.cc:1104-1131 */
  void Write_PowerSpectrum(std::string ofname) {
    detail::check(ctx_->get(), mf_grid_write_power_spectrum(handle(), ofname.c_str()), "Write_PowerSpectrum");
  }

  /* whole-field moves: the padded array of (n+2) n n reals; upload sets
   * the space the values belong to */
  void upload(const std::vector<real_t>& padded, space_t s) {
    if (padded.size() != stored_reals()) throw error(MF_ERR_SHAPE, "Grid_FFT::upload: size of the padded array");
    detail::check(ctx_->get(), mf_grid_upload(handle(), padded.data(), s == kspace_id ? MF_SPACE_K : MF_SPACE_R),
                  "mf_grid_upload");
  }
  void download(std::vector<real_t>& padded) const {
    padded.resize(stored_reals());
    detail::check(ctx_->get(), mf_grid_download(handle(), padded.data()), "mf_grid_download");
  }
  /* RNG_plugin::Fill_Grid (include/random_plugin.hh:37): n^3 real-space
   * float64 values, no padding */
  void fill_real64(const std::vector<double>& x) {
    if (x.size() != n_[0] * n_[0] * n_[0]) throw error(MF_ERR_SHAPE, "Grid_FFT::fill_real64: n^3 values");
    detail::check(ctx_->get(), mf_grid_fill_real64(handle(), x.data()), "mf_grid_fill_real64");
  }

  /* functions of the field on the host mirror (grid_fft.hh:450-810): the
   * field is read back, the functor runs per element on the host as in the
   * reference, and the result is written back in the grid's current space.
   * The pipeline's own k-space operators are CUDA kernels; these serve
   * arbitrary user functors. */
  template <typename F>
  void apply_function_k(const F& f) {
    each_k([&](size_t, size_t, size_t, size_t c, std::vector<real_t>& out) { put_c(out, c, f(get_c(out, c))); });
  }
  template <typename F>
  void apply_function_r(const F& f) {
    each_r([&](size_t, size_t, size_t, size_t r, std::vector<real_t>& out) { out[r] = f(out[r]); });
  }
  template <typename F>
  void apply_function_k_dep(const F& f) {
    each_k([&](size_t i, size_t j, size_t k, size_t c, std::vector<real_t>& out) {
      put_c(out, c, f(get_c(out, c), get_k<real_t>(i, j, k)));
    });
  }
  template <typename F>
  void apply_function_r_dep(const F& f) {
    each_r([&](size_t i, size_t j, size_t k, size_t r, std::vector<real_t>& out) {
      out[r] = f(out[r], get_r<real_t>(i, j, k));
    });
  }
  template <typename F, typename... G>
  void assign_function_of_grids_r(const F& f, G&... grids) {
    const auto in = read_all(grids...);
    each_r([&](size_t, size_t, size_t, size_t r, std::vector<real_t>& out) {
      out[r] = call_r(f, in, r, std::index_sequence_for<G...>{});
    });
  }
  template <typename F, typename... G>
  void assign_function_of_grids_k(const F& f, G&... grids) {
    const auto in = read_all(grids...);
    each_k([&](size_t, size_t, size_t, size_t c, std::vector<real_t>& out) {
      put_c(out, c, call_k(f, in, c, std::index_sequence_for<G...>{}));
    });
  }
  template <typename F, typename... G>
  void assign_function_of_grids_ijk(const F& f, G&... grids) {
    const auto in = read_all(grids...);
    each_k([&](size_t i, size_t j, size_t k, size_t c, std::vector<real_t>& out) {
      put_c(out, c, call_k(f, in, c, std::index_sequence_for<G...>{}, std::array<size_t, 3>{i, j, k}));
    });
  }
  template <typename F, typename... G>
  void assign_function_of_grids_kdep(const F& f, G&... grids) {
    const auto in = read_all(grids...);
    each_k([&](size_t i, size_t j, size_t k, size_t c, std::vector<real_t>& out) {
      put_c(out, c, call_k(f, in, c, std::index_sequence_for<G...>{}, get_k<real_t>(i, j, k)));
    });
  }

  /* single elements read from HBM (grid_fft.hh:179-211) */
  real_t relem(size_t i, size_t j, size_t k) const { return relem((i * n_[0] + j) * (n_[0] + 2) + k); }
  real_t relem(size_t idx) const {
    real_t v{};
    read(idx, stored_reals(), &v, sizeof v);
    return v;
  }
  ccomplex_t kelem(size_t i, size_t j, size_t k) const { return kelem((i * n_[0] + j) * (n_[0] / 2 + 1) + k); }
  ccomplex_t kelem(size_t idx) const {
    ccomplex_t v{};
    read(idx, stored_reals() / 2, &v, sizeof v);
    return v;
  }

 private:
  size_t stored_reals() const { return (n_[0] + 2) * n_[0] * n_[0]; }
  static ccomplex_t get_c(const std::vector<real_t>& a, size_t c) { return ccomplex_t(a[2 * c], a[2 * c + 1]); }
  static void put_c(std::vector<real_t>& a, size_t c, const ccomplex_t& v) {
    a[2 * c] = v.real();
    a[2 * c + 1] = v.imag();
  }
  /* loops of grid_fft.hh over sizes_[0..2] of the current space; B(i, j, k,
   * element index, padded array), then the array goes back to the device */
  template <typename B>
  void each_k(const B& body) {
    const space_t s = space();
    std::vector<real_t> out;
    download(out);
    const size_t n = n_[0], nk = n / 2 + 1;
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j)
        for (size_t k = 0; k < nk; ++k) body(i, j, k, (i * n + j) * nk + k, out);
    upload(out, s);
  }
  template <typename B>
  void each_r(const B& body) {
    const space_t s = space();
    std::vector<real_t> out;
    download(out);
    const size_t n = n_[0];
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j)
        for (size_t k = 0; k < n; ++k) body(i, j, k, (i * n + j) * (n + 2) + k, out);
    upload(out, s);
  }
  template <typename... G>
  static std::array<std::vector<real_t>, sizeof...(G)> read_all(G&... grids) {
    std::array<std::vector<real_t>, sizeof...(G)> in;
    size_t q = 0;
    (void)std::initializer_list<int>{(grids.download(in[q++]), 0)...};
    return in;
  }
  template <typename F, typename A, size_t... I, typename... Lead>
  static ccomplex_t call_k(const F& f, const A& in, size_t c, std::index_sequence<I...>, const Lead&... lead) {
    return ccomplex_t(f(lead..., get_c(in[I], c)...));
  }
  template <typename F, typename A, size_t... I>
  static real_t call_r(const F& f, const A& in, size_t r, std::index_sequence<I...>) {
    return real_t(f(in[I][r]...));
  }
  void read(size_t idx, size_t count, void* out, size_t bytes) const {
    if (idx >= count) throw std::out_of_range("Grid_FFT: element outside the stored layout");
    void* d = nullptr;
    detail::check(ctx_->get(), mf_grid_info(handle(), nullptr, nullptr, nullptr, &d, nullptr), "mf_grid_info");
    ctx_->synchronize();
    detail::check(ctx_->get(), mf_copy_to_host(out, static_cast<const char*>(d) + idx * bytes, bytes),
                  "mf_copy_to_host");
  }

  context* ctx_;
  std::array<size_t, 3> n_;
  std::array<real_t, 3> length_;
  space_t space0_;
  mf_grid* g_ = nullptr;
};

/* output operators (include/operators.hh:25-35): the target and the
 * operation the convolver applies in its last store */
namespace op {
struct output {
  mf_grid* target;
  int kind;
  double x;
};
template <typename field>
inline output assign_to(field& g) {
  return {g.handle(), MF_OP_ASSIGN, 1.0};
}
template <typename field, typename val>
inline output multiply_add_to(field& g, val x) {
  return {g.handle(), MF_OP_AXPY, static_cast<double>(x)};
}
template <typename field>
inline output add_to(field& g) {
  return {g.handle(), MF_OP_ADD, 1.0};
}
template <typename field>
inline output subtract_from(field& g) {
  return {g.handle(), MF_OP_SUB, 1.0};
}
}  // namespace op

/* BaseConvolver (include/convolution.hh:62-292): products of k-space
 * operator applications of two (or three) fields, the result handed to an
 * output operator.  Inputs are k-space grids. */
template <typename data_t>
class BaseConvolver {
 public:
  using real_t = data_t;
  using grid_t = Grid_FFT<data_t>;

  ~BaseConvolver() {
    if (cv_) mf_conv_destroy(cv_);
  }
  BaseConvolver(const BaseConvolver&) = delete;
  BaseConvolver& operator=(const BaseConvolver&) = delete;

  /* convolution.hh:74-103 */
  void convolve_Gradients(grid_t& inl, const std::array<int, 1>& d1l, grid_t& inr, const std::array<int, 1>& d1r,
                          op::output output_op) {
    conv2(opnd(inl, MF_OPND_GRAD, d1l[0]), opnd(inr, MF_OPND_GRAD, d1r[0]), output_op);
  }
  /* convolution.hh:105-134 */
  void convolve_Gradient_and_Hessian(grid_t& inl, const std::array<int, 1>& d1l, grid_t& inr,
                                     const std::array<int, 2>& d2r, op::output output_op) {
    conv2(opnd(inl, MF_OPND_GRAD, d1l[0]), opnd(inr, MF_OPND_HESS, d2r[0], d2r[1]), output_op);
  }
  /* convolution.hh:136-169 */
  void convolve_Hessians(grid_t& inl, const std::array<int, 2>& d2l, grid_t& inr, const std::array<int, 2>& d2r,
                         op::output output_op) {
    conv2(opnd(inl, MF_OPND_HESS, d2l[0], d2l[1]), opnd(inr, MF_OPND_HESS, d2r[0], d2r[1]), output_op);
  }
  /* convolution.hh:171-211 */
  void convolve_Hessians(grid_t& inl, const std::array<int, 2>& d2l, grid_t& inm, const std::array<int, 2>& d2m,
                         grid_t& inr, const std::array<int, 2>& d2r, op::output output_op) {
    const mf_operand a = opnd(inl, MF_OPND_HESS, d2l[0], d2l[1]), b = opnd(inm, MF_OPND_HESS, d2m[0], d2m[1]),
                     c = opnd(inr, MF_OPND_HESS, d2r[0], d2r[1]);
    detail::check(ctx_->get(), mf_conv_convolve3(cv_, &a, &b, &c, output_op.target, output_op.kind, output_op.x),
                  "convolve_Hessians");
  }
  /* convolution.hh:213-247 */
  void convolve_SumOfHessians(grid_t& inl, const std::array<int, 2>& d2l, grid_t& inr, const std::array<int, 2>& d2r1,
                              const std::array<int, 2>& d2r2, op::output output_op) {
    conv2(opnd(inl, MF_OPND_HESS, d2l[0], d2l[1]), opnd(inr, MF_OPND_SUM, d2r1[0], d2r1[1], d2r2[0], d2r2[1]),
          output_op);
  }
  /* convolution.hh:249-279 */
  void convolve_DifferenceOfHessians(grid_t& inl, const std::array<int, 2>& d2l, grid_t& inr,
                                     const std::array<int, 2>& d2r1, const std::array<int, 2>& d2r2,
                                     op::output output_op) {
    conv2(opnd(inl, MF_OPND_HESS, d2l[0], d2l[1]), opnd(inr, MF_OPND_DIFF, d2r1[0], d2r1[1], d2r2[0], d2r2[1]),
          output_op);
  }
  /* convolution.hh:281-292 */
  void multiply_field(grid_t& inl, grid_t& inr, op::output output_op) {
    conv2(opnd(inl, MF_OPND_PLAIN), opnd(inr, MF_OPND_PLAIN), output_op);
  }
  /* the last source term of a potential followed by
   * target.apply_InverseLaplacian(), in one call (src/ic_generator.cc:488,
   * 528, 545) */
  void convolve_Hessians_then_InverseLaplacian(grid_t& inl, const std::array<int, 2>& d2l, grid_t& inr,
                                               const std::array<int, 2>& d2r, op::output output_op) {
    const mf_operand a = opnd(inl, MF_OPND_HESS, d2l[0], d2l[1]), b = opnd(inr, MF_OPND_HESS, d2r[0], d2r[1]);
    detail::check(ctx_->get(), mf_conv_convolve2_invlap(cv_, &a, &b, output_op.target, output_op.kind, output_op.x),
                  "convolve_Hessians_then_InverseLaplacian");
  }

 protected:
  BaseConvolver(context& ctx, const std::array<size_t, 3>& N, const std::array<real_t, 3>& L, int kind) : ctx_(&ctx) {
    if (N[0] != N[1] || N[1] != N[2] || L[0] != L[1] || L[1] != L[2])
      throw error(MF_ERR_SHAPE, "convolver: cubic grids and boxes only");
    detail::check(ctx.get(),
                  mf_conv_create(ctx.get(), static_cast<int>(N[0]), static_cast<double>(L[0]),
                                 detail::prec_of<real_t>::value, kind, &cv_),
                  "mf_conv_create");
  }

 private:
  static mf_operand opnd(grid_t& g, int kind, int a = 0, int b = 0, int c = 0, int d = 0) {
    mf_operand o;
    o.grid = g.handle();
    o.kind = kind;
    o.d[0] = a;
    o.d[1] = b;
    o.d[2] = c;
    o.d[3] = d;
    return o;
  }
  void conv2(const mf_operand& a, const mf_operand& b, const op::output& o) {
    detail::check(ctx_->get(), mf_conv_convolve2(cv_, &a, &b, o.target, o.kind, o.x), "convolve");
  }

  context* ctx_;
  mf_conv* cv_ = nullptr;
};

/* OrszagConvolver (convolution.hh:429-669): 3/2-padded, dealiased */
template <typename data_t>
class OrszagConvolver : public BaseConvolver<data_t> {
 public:
  using real_t = data_t;
  OrszagConvolver(const std::array<size_t, 3>& N, const std::array<real_t, 3>& L)
      : OrszagConvolver(default_context(), N, L) {}
  OrszagConvolver(context& ctx, const std::array<size_t, 3>& N, const std::array<real_t, 3>& L)
      : BaseConvolver<data_t>(ctx, N, L, MF_CONV_ORSZAG) {}
};

/* NaiveConvolver (convolution.hh:296-426): unpadded, aliased */
template <typename data_t>
class NaiveConvolver : public BaseConvolver<data_t> {
 public:
  using real_t = data_t;
  NaiveConvolver(const std::array<size_t, 3>& N, const std::array<real_t, 3>& L)
      : NaiveConvolver(default_context(), N, L) {}
  NaiveConvolver(context& ctx, const std::array<size_t, 3>& N, const std::array<real_t, 3>& L)
      : BaseConvolver<data_t>(ctx, N, L, MF_CONV_NAIVE) {}
};

}  // namespace mfgpu

#endif /* MONOFONIC_GB300_HPP */
