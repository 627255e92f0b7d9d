// LPT pipeline of ic_generator::run (src/ic_generator.cc:90-948) on one
// device: white noise -> phi(1) -> phi(2), phi(3), A(3) through the fused
// Orszag convolver -> displacement/velocity assembly -> lattice positions,
// velocities and particle IDs.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/monofonic_gb300_ic.h"
#include "mf_cosmo.h"
#include "mf_eh.cuh"
#include "mf_runtime.h"

namespace mf {
namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(size_t n, int per = 4) {
  size_t b = (n + (size_t)kThreads * per - 1) / ((size_t)kThreads * per);
  if (b > 152u * 32u) b = 152u * 32u;
  return (unsigned)(b ? b : 1);
}

// amplitude table amp(k2) = k^{n_s/2} T(k) sqrt(pnorm), k = sqrt(k2)*kfac
// (get_amplitude, include/cosmology_calculator.hh:405-408), FP64
__global__ void k_amp_table(double* amp, int nk2, double kfac, double half_ns, double sqrtpnorm, EHParams eh,
                            const double* tk) {
  for (int k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 < nk2; k2 += gridDim.x * blockDim.x) {
    const double k = sqrt((double)k2) * kfac;
    const double t = tk ? tk[k2] : eh_eval(eh, k);
    amp[k2] = pow(k, half_ns) * t * sqrtpnorm;
  }
}

// noise normalisation (ic_generator.cc:341-346) in place, then
// phi = -wn amp(k) / k^2 with zero DC (ic_generator.cc:449-457)
template <typename T>
__global__ void k_phi1(cplx<T>* wn, cplx<T>* phi, int n, double kfac, const double* amp, double sign_over_volfac,
                       int fixing) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const int ii = i - (i > n / 2 ? n : 0), jj = j - (j > n / 2 ? n : 0);
    cplx<T> w = wn[idx];
    if (fixing) {
      const T a = sqrt(w.x * w.x + w.y * w.y);
      if (a != T(0)) w = mkc<T>(w.x / a, w.y / a);
    }
    w = mkc<T>(w.x * T(sign_over_volfac), w.y * T(sign_over_volfac));
    wn[idx] = w;
    const T kx = T(ii) * T(kfac), ky = T(jj) * T(kfac), kk = T(kz) * T(kfac);
    const T kmod = sqrt(kx * kx + ky * ky + kk * kk);
    const int k2 = ii * ii + jj * jj + kz * kz;
    const T a = T(amp[k2]);
    const T den = kmod * kmod;
    phi[idx] = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(-(w.x * a) / den, -(w.y * a) / den);
  }
}

struct AssembleArgs {
  const void* phi;
  const void* phi2;
  const void* phi3;
  const void* A3[3];
  int order;
  int d;          // component
  double w1, w2, w3, w3c;  // g_n (positions) or vfac_n g_n (velocities) and the A3 weight
  double unit_over_L;
  int shift;      // multiply by exp(i s.k dx)
  double s[3];
  double dx;
};

// k-space displacement/velocity combination (ic_generator.cc:829-858,
// :884-931) with the growth-factor-weighted order sum in FP64, times
// unit/L, zero DC; optional sub-lattice phase of shift_field
// (grid_fft.hh:832-842) folded in
template <typename T>
__global__ void k_assemble(AssembleArgs a, cplx<T>* out, int n, double kfac) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  const cplx<T>* P1 = (const cplx<T>*)a.phi;
  const cplx<T>* P2 = (const cplx<T>*)a.phi2;
  const cplx<T>* P3 = (const cplx<T>*)a.phi3;
  const int dp = (a.d + 1) % 3, dpp = (a.d + 2) % 3;
  const cplx<T>* Adp = (const cplx<T>*)a.A3[dp];
  const cplx<T>* Adpp = (const cplx<T>*)a.A3[dpp];
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const int ijk[3] = {i, j, kz};
    const double gd = gradk<double>(ijk[a.d], n, kfac);
    cplx<T> v = P1[idx];
    double tr = a.w1 * (double)v.x, ti = a.w1 * (double)v.y;
    if (a.order > 1) {
      v = P2[idx];
      tr += a.w2 * (double)v.x;
      ti += a.w2 * (double)v.y;
    }
    if (a.order > 2) {
      v = P3[idx];
      tr += a.w3 * (double)v.x;
      ti += a.w3 * (double)v.y;
    }
    // i g_d * phitot
    double rr = -gd * ti, ri = gd * tr;
    if (a.order > 2) {
      const double gp = gradk<double>(ijk[dp], n, kfac), gpp = gradk<double>(ijk[dpp], n, kfac);
      const cplx<T> x1 = Adpp[idx], x2 = Adp[idx];
      // i g_p A3[pp] - i g_pp A3[p], A3 scaled by w3c
      const double ar = a.w3c * (-(gp * (double)x1.y) + gpp * (double)x2.y);
      const double ai = a.w3c * (gp * (double)x1.x - gpp * (double)x2.x);
      rr += ar;
      ri += ai;
    }
    rr *= a.unit_over_L;
    ri *= a.unit_over_L;
    if (idx == 0) { rr = 0; ri = 0; }
    if (a.shift) {
      const double sh = a.s[0] * kcomp<double>(i, n, kfac) * a.dx + a.s[1] * kcomp<double>(j, n, kfac) * a.dx +
                        a.s[2] * kcomp<double>(kz, n, kfac) * a.dx;
      double sn, cs;
      sincos(sh, &sn, &cs);
      const double nr = rr * cs - ri * sn, ni = rr * sn + ri * cs;
      rr = nr;
      ri = ni;
    }
    out[idx] = mkc<T>(T(rr), T(ri));
  }
}

// lattice readout (set_positions / set_velocities, particle_generator.hh:499-639)
template <typename T, typename P>
__global__ void k_lattice(const T* psi, int n, P* dst, int d, int ishift, double sd, double lunit, int with_q,
                          int fields_mode) {
  const size_t n3 = (size_t)n * n * n;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const size_t line = c / n;
    const int k = (int)(c % n);
    const double v = (double)psi[line * (n + 2) + k];
    if (fields_mode) {
      dst[(size_t)d * n3 + c] = (P)v;
      continue;
    }
    double out = v;
    if (with_q) {
      const int j = (int)(line % n), i = (int)(line / n);
      const int idx = (d == 0) ? i : (d == 1) ? j : k;
      out = ((double)idx + sd) / (double)n * lunit + v;
    }
    dst[3 * ((size_t)ishift * n3 + c) + d] = (P)out;
  }
}

template <typename I>
__global__ void k_ids(I* ids, int n, int overload, uint64_t offset) {
  const size_t n3 = (size_t)n * n * n;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x)
    for (int il = 0; il < overload; ++il) ids[(size_t)il * n3 + c] = (I)(offset + (uint64_t)overload * c + il);
}

// lattice shifts (particle_generator.hh:47-54)
const double kShifts[4][8][3] = {
    {{0, 0, 0}},
    {{0, 0, 0}, {0.5, 0.5, 0.5}},
    {{0, 0, 0}, {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}},
    {{0, 0, 0}, {0, 0, 0.5}, {0, 0.5, 0}, {0, 0.5, 0.5}, {0.5, 0, 0}, {0.5, 0, 0.5}, {0.5, 0.5, 0}, {0.5, 0.5, 0.5}},
};

}  // namespace
}  // namespace mf

using namespace mf;

struct mf_ic {
  mf_ctx* ctx = nullptr;
  mf_ic_params p{};
  mf_grid* wn = nullptr;
  mf_grid* f[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // phi, phi2, phi3, A3x, A3y, A3z
  mf_grid* tmp = nullptr;
  mf_conv* conv = nullptr;
  double* amp = nullptr;
  int nk2 = 0;
  void* dpos = nullptr;
  void* dvel = nullptr;
  void* dids = nullptr;
  size_t pos_bytes = 0, vel_bytes = 0, id_bytes = 0;
  int64_t npart = 0;
  cudaEvent_t ev[9] = {};
  bool noise_set = false;
};

namespace {

int check_params(const mf_ic_params* p) {
  if (!p) return MF_ERR_ARG;
  if (!grid_size_supported(p->ngrid)) return MF_ERR_SHAPE;
  if (p->lpt_order < 1 || p->lpt_order > 3) return MF_ERR_ARG;
  if (p->lattice < MF_LATTICE_SC || p->lattice > MF_LATTICE_RSC) return MF_ERR_ARG;
  if (p->precision != MF_PREC_F64 && p->precision != MF_PREC_F32) return MF_ERR_ARG;
  if (p->convolver != MF_CONV_ORSZAG && p->convolver != MF_CONV_NAIVE) return MF_ERR_ARG;
  if (p->out_kind != MF_OUT_PARTICLES && p->out_kind != MF_OUT_FIELDS) return MF_ERR_ARG;
  if (p->out_kind == MF_OUT_FIELDS && p->lattice != MF_LATTICE_SC) return MF_ERR_ARG;
  if (!(p->boxlen > 0)) return MF_ERR_ARG;
  if (p->plt) return MF_ERR_ARG;  // PLT tables are built by mf_ic_create when supported
  return MF_OK;
}

void output_sizes(const mf_ic_params* p, int64_t* np, size_t* pb, size_t* vb, size_t* ib) {
  const int64_t n3 = (int64_t)p->ngrid * p->ngrid * p->ngrid;
  const int overload = 1 << p->lattice;
  if (p->out_kind == MF_OUT_FIELDS) {
    *np = n3;
    *pb = *vb = (size_t)3 * n3 * sizeof(double);
    *ib = 0;
    return;
  }
  *np = n3 * overload;
  const size_t rs = p->pos64 ? 8 : 4;
  *pb = *vb = (size_t)3 * (*np) * rs;
  *ib = (size_t)(*np) * (p->id64 ? 8 : 4);
}

template <typename T>
int run_impl(mf_ic* ic, mf_particles* out) {
  mf_ctx* c = ic->ctx;
  cudaStream_t s = c->stream;
  const mf_ic_params& p = ic->p;
  const int n = p.ngrid, Kz = n / 2 + 1;
  const double L = p.boxlen, kfac = 2.0 * M_PI / L;
  const size_t nk = (size_t)n * n * Kz;
  cudaError_t e;
#define CK(x)                                            \
  do {                                                   \
    e = (x);                                             \
    if (e != cudaSuccess) return cuda_err(c, e, #x);     \
  } while (0)

  CK(cudaEventRecord(ic->ev[0], s));
  // ---- white noise to k-space, phi(1) -----------------------------------
  CK(fft3d_r2c<T>(c, (T*)ic->wn->d, n));
  ic->wn->space = MF_SPACE_K;
  {
    EHParams eh;
    eh_setup(p.cosmo.H0 > 0 ? p.cosmo.H0 : 100.0 * p.cosmo.h, p.cosmo.Omega_m, p.cosmo.Omega_b, p.cosmo.Tcmb, &eh);
    const double* tk = nullptr;
    if (p.tk_table) {
      CK(cudaMemcpyAsync(ic->amp + ic->nk2, p.tk_table, sizeof(double) * ic->nk2, cudaMemcpyHostToDevice, s));
      tk = ic->amp + ic->nk2;
    }
    LaunchScope ls0(c, KK_POINTWISE);
    k_amp_table<<<(ic->nk2 + 255) / 256, 256, 0, s>>>(ic->amp, ic->nk2, kfac, 0.5 * p.cosmo.n_s,
                                                       std::sqrt(p.cosmo.pnorm), eh, tk);
    CK(cudaGetLastError());
    const double volfac = std::pow(L / n / 2.0 / M_PI, 1.5);
    const double sgn = (p.inversion ? -1.0 : 1.0) / volfac;
    LaunchScope ls1(c, KK_POINTWISE);
    k_phi1<T><<<blocks_for(nk), kThreads, 0, s>>>((cplx<T>*)ic->wn->d, (cplx<T>*)ic->f[0]->d, n, kfac, ic->amp, sgn,
                                                   p.fixing);
    CK(cudaGetLastError());
    ic->f[0]->space = MF_SPACE_K;
  }
  CK(cudaEventRecord(ic->ev[1], s));

  auto H = [&](int g, int a, int b) {
    Operand<T> o{};
    o.f = (const cplx<T>*)ic->f[g]->d;
    o.kind = OPND_HESS;
    o.d[0] = a; o.d[1] = b;
    return o;
  };
  auto S = [&](int g, int a, int b, int cc, int d, bool diff) {
    Operand<T> o{};
    o.f = (const cplx<T>*)ic->f[g]->d;
    o.kind = diff ? OPND_DIFF : OPND_SUM;
    o.d[0] = a; o.d[1] = b; o.d[2] = cc; o.d[3] = d;
    return o;
  };
  auto conv2 = [&](Operand<T> A, Operand<T> B, int tgt, int op, double x, int invlap) -> cudaError_t {
    Operand<T> o[2] = {A, B};
    return conv_run<T>(ic->conv, o, 2, (cplx<T>*)ic->f[tgt]->d, op, T(x), invlap);
  };
  const bool orszag = p.convolver == MF_CONV_ORSZAG;
  auto conv3 = [&](Operand<T> A, Operand<T> B, Operand<T> C3, int tgt, int op, double x) -> cudaError_t {
    if (!orszag) {
      Operand<T> o[3] = {A, B, C3};
      return conv_run<T>(ic->conv, o, 3, (cplx<T>*)ic->f[tgt]->d, op, T(x), 0);
    }
    Operand<T> o[2] = {A, B};
    cudaError_t e2 = conv_run<T>(ic->conv, o, 2, (cplx<T>*)ic->conv->fbuf->d, OUT_ASSIGN, T(1), 0);
    if (e2 != cudaSuccess) return e2;
    Operand<T> f{};
    f.f = (const cplx<T>*)ic->conv->fbuf->d;
    f.kind = OPND_PLAIN;
    Operand<T> o2[2] = {f, C3};
    return conv_run<T>(ic->conv, o2, 2, (cplx<T>*)ic->f[tgt]->d, op, T(x), 0);
  };

  // ---- phi(2) (ic_generator.cc:471-488) ----------------------------------
  if (p.lpt_order > 1) {
    CK(conv2(H(0, 0, 0), S(0, 1, 1, 2, 2, false), 1, OUT_ASSIGN, 1, 0));
    CK(conv2(H(0, 1, 1), H(0, 2, 2), 1, OUT_ADD, 1, 0));
    CK(conv2(H(0, 0, 1), H(0, 0, 1), 1, OUT_SUB, 1, 0));
    CK(conv2(H(0, 0, 2), H(0, 0, 2), 1, OUT_SUB, 1, 0));
    CK(conv2(H(0, 1, 2), H(0, 1, 2), 1, OUT_SUB, 1, 1));
    ic->f[1]->space = MF_SPACE_K;
  }
  CK(cudaEventRecord(ic->ev[2], s));
  // ---- phi(3) (ic_generator.cc:511-528) ----------------------------------
  if (p.lpt_order > 2) {
    CK(conv3(H(0, 0, 0), H(0, 1, 1), H(0, 2, 2), 2, OUT_ASSIGN, 1));
    CK(conv3(H(0, 0, 1), H(0, 0, 2), H(0, 1, 2), 2, OUT_AXPY, 2.0));
    CK(conv3(H(0, 1, 2), H(0, 1, 2), H(0, 0, 0), 2, OUT_SUB, 1));
    CK(conv3(H(0, 0, 2), H(0, 0, 2), H(0, 1, 1), 2, OUT_SUB, 1));
    CK(conv3(H(0, 0, 1), H(0, 0, 1), H(0, 2, 2), 2, OUT_SUB, 1));
    CK(conv2(H(0, 0, 0), S(1, 1, 1, 2, 2, false), 2, OUT_AXPY, -5.0 / 7.0, 0));
    CK(conv2(H(0, 1, 1), S(1, 2, 2, 0, 0, false), 2, OUT_AXPY, -5.0 / 7.0, 0));
    CK(conv2(H(0, 2, 2), S(1, 0, 0, 1, 1, false), 2, OUT_AXPY, -5.0 / 7.0, 0));
    CK(conv2(H(0, 0, 1), H(1, 0, 1), 2, OUT_AXPY, +10.0 / 7.0, 0));
    CK(conv2(H(0, 0, 2), H(1, 0, 2), 2, OUT_AXPY, +10.0 / 7.0, 0));
    CK(conv2(H(0, 1, 2), H(1, 1, 2), 2, OUT_AXPY, +10.0 / 7.0, 1));
    ic->f[2]->space = MF_SPACE_K;
  }
  CK(cudaEventRecord(ic->ev[3], s));
  // ---- A(3) (ic_generator.cc:534-545) -----------------------------------
  if (p.lpt_order > 2) {
    for (int d = 0; d < 3; ++d) {
      const int dp = (d + 1) % 3, dpp = (d + 2) % 3, tg = 3 + d;
      CK(conv2(H(1, d, dp), H(0, d, dpp), tg, OUT_ASSIGN, 1, 0));
      CK(conv2(H(1, d, dpp), H(0, d, dp), tg, OUT_SUB, 1, 0));
      CK(conv2(H(0, dp, dpp), S(1, dp, dp, dpp, dpp, true), tg, OUT_ADD, 1, 0));
      CK(conv2(H(1, dp, dpp), S(0, dp, dp, dpp, dpp, true), tg, OUT_SUB, 1, 1));
      ic->f[tg]->space = MF_SPACE_K;
    }
  }
  CK(cudaEventRecord(ic->ev[4], s));

  // ---- growth factors (ic_generator.cc:221-234) ---------------------------
  const double D = p.cosmo.Dplus;
  const double g1 = -D;
  const double g2 = (p.lpt_order > 1) ? -3.0 / 7.0 * D * D : 0.0;
  const double g3 = (p.lpt_order > 2) ? 1.0 / 3.0 * D * D * D : 0.0;
  const double g3c = (p.lpt_order > 2) ? 1.0 / 7.0 * D * D * D : 0.0;
  const double vf = p.cosmo.vfac;
  const int overload = 1 << p.lattice;
  const bool fields = p.out_kind == MF_OUT_FIELDS;

  AssembleArgs a{};
  a.phi = ic->f[0]->d;
  a.phi2 = ic->f[1] ? ic->f[1]->d : nullptr;
  a.phi3 = ic->f[2] ? ic->f[2]->d : nullptr;
  for (int d = 0; d < 3; ++d) a.A3[d] = ic->f[3 + d] ? ic->f[3 + d]->d : nullptr;
  a.order = p.lpt_order;
  a.dx = L / n;
  T* tmpr = (T*)ic->tmp->d;
  for (int pass = 0; pass < 2; ++pass) {  // 0: positions, 1: velocities
    const bool vel = pass == 1;
    // weights: positions g_n; velocities vfac_n g_n with vfac_n = n vfac
    a.w1 = vel ? vf * g1 : g1;
    a.w2 = vel ? 2 * vf * g2 : g2;
    a.w3 = vel ? 3 * vf * g3 : g3;
    a.w3c = vel ? 3 * vf * g3c : g3c;
    a.unit_over_L = (vel ? p.vunit : p.lunit) / L;
    void* dst = vel ? ic->dvel : ic->dpos;
    for (int d = 0; d < 3; ++d) {
      a.d = d;
      for (int ish = 0; ish < overload; ++ish) {
        a.shift = ish > 0;
        for (int q = 0; q < 3; ++q) a.s[q] = kShifts[p.lattice][ish][q];
        {
          LaunchScope ls(c, KK_POINTWISE);
          k_assemble<T><<<blocks_for(nk), kThreads, 0, s>>>(a, (cplx<T>*)tmpr, n, kfac);
        }
        CK(cudaGetLastError());
        CK(fft3d_c2r<T>(c, tmpr, n));
        const size_t n3 = (size_t)n * n * n;
        const double sd = kShifts[p.lattice][ish][d];
        LaunchScope ls(c, KK_POINTWISE);
        if (fields) {
          k_lattice<T, double><<<blocks_for(n3), kThreads, 0, s>>>(tmpr, n, (double*)dst, d, 0, 0.0, 0.0, 0, 1);
        } else if (p.pos64) {
          k_lattice<T, double><<<blocks_for(n3), kThreads, 0, s>>>(tmpr, n, (double*)dst, d, ish, sd, p.lunit,
                                                                  vel ? 0 : 1, 0);
        } else {
          k_lattice<T, float><<<blocks_for(n3), kThreads, 0, s>>>(tmpr, n, (float*)dst, d, ish, sd, p.lunit,
                                                                 vel ? 0 : 1, 0);
        }
        CK(cudaGetLastError());
      }
    }
    CK(cudaEventRecord(ic->ev[5 + pass], s));
  }
  // ---- particle IDs (particle_generator.hh:212-253) ------------------------
  if (!fields) {
    LaunchScope ls(c, KK_POINTWISE);
    if (p.id64)
      k_ids<uint64_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint64_t*)ic->dids, n, overload, 0);
    else
      k_ids<uint32_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint32_t*)ic->dids, n, overload, 0);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(ic->ev[7], s));
  // ---- hand-off ---------------------------------------------------------------
  if (out) {
    out->npart = ic->npart;
    if (out->location == MF_LOC_HOST) {
      if (!out->pos || !out->vel || (!fields && !out->ids)) return set_err(c, MF_ERR_ARG, "mf_ic_run: null host buffer");
      CK(cudaMemcpyAsync(out->pos, ic->dpos, ic->pos_bytes, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(out->vel, ic->dvel, ic->vel_bytes, cudaMemcpyDeviceToHost, s));
      if (!fields) CK(cudaMemcpyAsync(out->ids, ic->dids, ic->id_bytes, cudaMemcpyDeviceToHost, s));
    } else {
      out->pos = ic->dpos;
      out->vel = ic->dvel;
      out->ids = ic->dids;
    }
  }
  CK(cudaEventRecord(ic->ev[8], s));
  CK(cudaStreamSynchronize(s));
#undef CK
  return MF_OK;
}

}  // namespace

extern "C" int mf_ic_output_size(const mf_ic_params* p, int64_t* np, size_t* pb, size_t* vb, size_t* ib) {
  int rc = check_params(p);
  if (rc) return rc;
  int64_t a; size_t b, c2, d;
  output_sizes(p, &a, &b, &c2, &d);
  if (np) *np = a;
  if (pb) *pb = b;
  if (vb) *vb = c2;
  if (ib) *ib = d;
  return MF_OK;
}

extern "C" int mf_ic_device_footprint(const mf_ic_params* p, size_t* bytes) {
  int rc = check_params(p);
  if (rc) return rc;
  if (!bytes) return MF_ERR_ARG;
  const int n = p->ngrid;
  const size_t ps = p->precision == MF_PREC_F32 ? 4 : 8;
  const size_t grid = grid_reals(n) * ps;
  int ngrids = 3 + (p->lpt_order > 1 ? 1 : 0) + (p->lpt_order > 2 ? 4 : 0);
  size_t conv = 0;
  if (p->lpt_order > 1) {
    const size_t M = (p->convolver == MF_CONV_ORSZAG) ? 3 * n / 2 : n;
    const int nbuf = (p->convolver == MF_CONV_ORSZAG) ? 2 : 3;
    conv = (size_t)nbuf * M * M * (n / 2 + 1) * 2 * ps + (p->convolver == MF_CONV_ORSZAG ? grid : 0);
  }
  int64_t np; size_t pb, vb, ib;
  output_sizes(p, &np, &pb, &vb, &ib);
  const size_t nk2 = 3 * (size_t)(n / 2) * (n / 2) + 1;
  *bytes = ngrids * grid + conv + pb + vb + ib + 2 * nk2 * sizeof(double);
  return MF_OK;
}

extern "C" int mf_ic_destroy(mf_ic* ic) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (ic->wn) mf_grid_destroy(ic->wn);
  for (auto& g : ic->f)
    if (g) mf_grid_destroy(g);
  if (ic->tmp) mf_grid_destroy(ic->tmp);
  if (ic->conv) mf_conv_destroy(ic->conv);
  cudaFree(ic->amp);
  cudaFree(ic->dpos);
  cudaFree(ic->dvel);
  cudaFree(ic->dids);
  for (auto& e : ic->ev)
    if (e) cudaEventDestroy(e);
  --c->children;
  delete ic;
  return MF_OK;
}

extern "C" int mf_ic_create(mf_ctx* c, const mf_ic_params* p, mf_ic** out) {
  if (!c || !out) return MF_ERR_ARG;
  *out = nullptr;
  int rc = check_params(p);
  if (rc) return set_err(c, rc, "mf_ic_create: invalid parameters");
  cudaSetDevice(c->device);
  mf_ic* ic = new (std::nothrow) mf_ic();
  if (!ic) return MF_ERR_OOM;
  ic->ctx = c;
  ++c->children;
  ic->p = *p;
  ic->p.tk_table = nullptr;
  const int n = p->ngrid;
  auto fail = [&](int code) { mf_ic_destroy(ic); return code; };
  if ((rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_R, &ic->wn))) return fail(rc);
  const int nf = (p->lpt_order > 2) ? 6 : p->lpt_order;
  for (int i = 0; i < nf; ++i)
    if ((rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &ic->f[i]))) return fail(rc);
  if ((rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &ic->tmp))) return fail(rc);
  if (p->lpt_order > 1)
    if ((rc = mf_conv_create(c, n, p->boxlen, p->precision, p->convolver, &ic->conv))) return fail(rc);
  ic->nk2 = 3 * (n / 2) * (n / 2) + 1;
  cudaError_t e = cudaMalloc(&ic->amp, sizeof(double) * 2 * ic->nk2);
  if (e != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: amplitude table"));
  output_sizes(p, &ic->npart, &ic->pos_bytes, &ic->vel_bytes, &ic->id_bytes);
  if ((e = cudaMalloc(&ic->dpos, ic->pos_bytes)) != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: positions"));
  if ((e = cudaMalloc(&ic->dvel, ic->vel_bytes)) != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: velocities"));
  if (ic->id_bytes && (e = cudaMalloc(&ic->dids, ic->id_bytes)) != cudaSuccess)
    return fail(cuda_err(c, e, "mf_ic_create: ids"));
  for (auto& ev : ic->ev)
    if ((e = cudaEventCreate(&ev)) != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: events"));
  *out = ic;
  return MF_OK;
}

extern "C" int mf_ic_set_noise(mf_ic* ic, const double* noise, int location) {
  if (!ic || !noise) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  cudaSetDevice(c->device);
  const int n = ic->p.ngrid;
  const size_t n3 = (size_t)n * n * n;
  cudaError_t e = cudaSuccess;
  if (location == MF_LOC_HOST) {
    double* stage = nullptr;
    e = cudaMallocAsync(&stage, n3 * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(stage, noise, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = (ic->p.precision == MF_PREC_F64) ? pw_fill_from_f64<double>((double*)ic->wn->d, stage, n, c->stream)
                                           : pw_fill_from_f64<float>((float*)ic->wn->d, stage, n, c->stream);
    if (stage) cudaFreeAsync(stage, c->stream);
  } else {
    e = (ic->p.precision == MF_PREC_F64) ? pw_fill_from_f64<double>((double*)ic->wn->d, noise, n, c->stream)
                                         : pw_fill_from_f64<float>((float*)ic->wn->d, noise, n, c->stream);
  }
  if (e != cudaSuccess) return cuda_err(c, e, "mf_ic_set_noise");
  ic->wn->space = MF_SPACE_R;
  ic->noise_set = true;
  return MF_OK;
}

extern "C" int mf_ic_run(mf_ic* ic, mf_particles* out) {
  if (!ic) return MF_ERR_ARG;
  if (!ic->noise_set) return set_err(ic->ctx, MF_ERR_STATE, "mf_ic_run: white noise not set");
  cudaSetDevice(ic->ctx->device);
  const int rc = (ic->p.precision == MF_PREC_F64) ? run_impl<double>(ic, out) : run_impl<float>(ic, out);
  ic->noise_set = false;  // the noise grid is consumed (transformed and normalised in place)
  return rc;
}

extern "C" int mf_ic_stage_times(const mf_ic* ic, double* ms) {
  if (!ic || !ms) return MF_ERR_ARG;
  for (int i = 0; i < 8; ++i) {
    float t = 0;
    if (cudaEventElapsedTime(&t, ic->ev[i], ic->ev[i + 1]) != cudaSuccess) t = -1;
    ms[i] = t;
  }
  return MF_OK;
}

extern "C" int mf_ic_get_potential(mf_ic* ic, int which, mf_grid** out) {
  if (!ic || !out || which < 0 || which > 5 || !ic->f[which]) return MF_ERR_ARG;
  *out = ic->f[which];
  return MF_OK;
}

extern "C" int mf_ic_get_noise(mf_ic* ic, mf_grid** out) {
  if (!ic || !out) return MF_ERR_ARG;
  *out = ic->wn;
  return MF_OK;
}
