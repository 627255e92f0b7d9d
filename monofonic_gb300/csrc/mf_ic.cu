// LPT pipeline of ic_generator::run (src/ic_generator.cc:90-948) on one
// device: white noise -> phi(1) -> phi(2), phi(3), A(3) through the fused
// Orszag convolver -> displacement/velocity assembly -> lattice positions,
// velocities and particle IDs.
#include <algorithm>
#include <cmath>
#include <initializer_list>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/monofonic_gb300_ic.h"
#include "mf_cosmo.h"
#include "mf_eh.cuh"
#include "mf_plt.h"
#include "mf_ppt.h"
#include "mf_runtime.h"

// host hand-off during a run (a build-time knob).  The IDs are copied while
// the run computes either way; 1 streams every sub-lattice slice of the
// positions and velocities as soon as each is final (the copies queue on one
// copy engine, so the tail after the last kernel is one slice); 0 copies the
// positions during the velocity pass and the velocities after it
#ifndef MF_STREAM_HANDOFF
#define MF_STREAM_HANDOFF 1
#endif

namespace mf {
namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(size_t n, int per = 4) {
  size_t b = (n + (size_t)kThreads * per - 1) / ((size_t)kThreads * per);
  if (b > 152u * 32u) b = 152u * 32u;
  return (unsigned)(b ? b : 1);
}

// per-run parameters the kernels read from device memory, so that a pipeline
// recorded once into a CUDA graph replays with a new cosmology and seed
struct ICDyn {
  EHParams eh;              // TFset_parameters of the cosmology
  double half_ns, sqrtpnorm;
  double w[2][4];           // positions / velocities: weights of phi, phi2, phi3 and the A3 term
  unsigned long long seed;  // white-noise seed (device generator)
  // two species (ic_generator.cc:157-166, :615-619): C_species, Omega_species,
  // the theta_bc weight of the velocities (-vfac C_species, 0 without the
  // relative-velocity mode), D+_target and sqrt(D+_target / D+_start)
  double Cs[2], Omega_s[2], wbc[2];
  double bc_Dt, bc_sqrtDr;
  int vrel;
};

// amplitudes of the baryon-CDM modes per integer k^2: get_amplitude_delta_bc
// and get_amplitude_theta_bc (cosmology_calculator.hh:416-431) from the host
// tables of T_delta_bc and T_theta_bc (zero where a table is absent)
__global__ void k_amp_bc(double* ampd, double* ampt, double* ampd0, int nk2, double kfac, const ICDyn* __restrict__ dyn,
                         const double* tdbc, const double* ttbc) {
  const double half_ns = dyn->half_ns, sqrtpnorm = dyn->sqrtpnorm, Dt = dyn->bc_Dt, sDr = dyn->bc_sqrtDr;
  const int vrel = dyn->vrel;
  for (int k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 < nk2; k2 += gridDim.x * blockDim.x) {
    const double k = sqrt((double)k2) * kfac;
    const double td = tdbc ? tdbc[k2] : 0.0, tt = ttbc ? ttbc[k2] : 0.0;
    const double dbc = td + (vrel ? 2 * tt * (sDr - 1.0) : 0.0);
    ampd[k2] = pow(k, half_ns) * dbc * (sqrtpnorm * Dt);
    ampt[k2] = vrel ? pow(k, half_ns) * (tt * sDr) * (sqrtpnorm * Dt) : 0.0;
    ampd0[k2] = pow(k, half_ns) * td * (sqrtpnorm * Dt);  // without the relative-velocity mode
  }
}

// baryon-CDM fields from the normalised noise: rho_bc = wn amp_dbc
// (ic_generator.cc:655-660) and the relative-velocity potential
// psi_bc = amp_tbc wn / k^2 (ic_generator.cc:907-910), both with zero DC
template <typename T>
__global__ void k_bc_fields(const cplx<T>* wn, cplx<T>* rho, cplx<T>* psi, cplx<T>* rho0, int n, double kfac,
                            const double* ampd, const double* ampt, const double* ampd0) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    const int ii = i - (i > n / 2 ? n : 0), jj = j - (j > n / 2 ? n : 0);
    const int k2 = ii * ii + jj * jj + kz * kz;
    const cplx<T> w = wn[idx];
    if (rho) {
      const T a = T(ampd[k2]);
      rho[idx] = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(w.x * a, w.y * a);
    }
    if (rho0) {  // the Eulerian branch's delta_bc (ic_generator.cc:685-688)
      const T a = T(ampd0[k2]);
      rho0[idx] = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(w.x * a, w.y * a);
    }
    if (psi) {
      const T kx = T(ii) * T(kfac), ky = T(jj) * T(kfac), kk = T(kz) * T(kfac);
      const T kn2 = kx * kx + ky * ky + kk * kk;
      const T a = T(ampt[k2]);
      psi[idx] = (idx == 0) ? mkc<T>(T(0), T(0)) : mkc<T>(w.x * a / kn2, w.y * a / kn2);
    }
  }
}

// one shift_field chain over a k-space grid (set_masses, particle_generator.hh:389-401)
template <typename T>
__global__ void k_shift_chain(const cplx<T>* src, cplx<T>* dst, int n, ShiftChain<T> ch) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    cplx<T> v[1] = {src[idx]};
    cplx<T> vm[1] = {mkc<T>(T(0), T(0))};
    if (kz == 0 || kz == n / 2) vm[0] = src[((size_t)((n - i) % n) * n + (n - j) % n) * Kz + kz];
    ch.template apply<1>(n, i, j, kz, v, vm);
    dst[idx] = v[0];
  }
}

// set_masses (particle_generator.hh:369-422): particle ip = ishift*n^3 + cell
// gets pmeanmass * (1 + C_s delta_bc) Omega_s munit (ic_generator.cc:662-664),
// delta_bc read from the shifted real field (padded rows), or 0
template <typename T, typename P>
__global__ void k_masses(P* mass, const T* delta, int n, int ishift, double pmean, double munit,
                         const ICDyn* __restrict__ dyn, int species) {
  const size_t n3 = (size_t)n * n * n;
  const double C = dyn->Cs[species], Om = dyn->Omega_s[species];
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const size_t i = c / ((size_t)n * n), j = (c / n) % n, k = c % n;
    const double v = delta ? (double)delta[(i * n + j) * (n + 2) + k] : 0.0;
    const double rho = (1.0 + C * v) * Om * munit;
    mass[(size_t)ishift * n3 + c] = (P)(pmean * rho);
  }
}

// amplitude table amp(k2) = k^{n_s/2} T(k) sqrt(pnorm), k = sqrt(k2)*kfac
// (get_amplitude, include/cosmology_calculator.hh:405-408), FP64
__global__ void k_amp_table(double* amp, int nk2, double kfac, const ICDyn* __restrict__ dyn, const double* tk) {
  const double half_ns = dyn->half_ns, sqrtpnorm = dyn->sqrtpnorm;
  for (int k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 < nk2; k2 += gridDim.x * blockDim.x) {
    const double k = sqrt((double)k2) * kfac;
    const double t = tk ? tk[k2] : eh_eval(dyn->eh, k);
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

// growth-factor-weighted sum of the orders (ic_generator.cc:550-563 and
// :835-845 / :889-899) in FP64, stored in the grid precision
template <typename T>
__global__ void k_phitot(cplx<T>* out, const cplx<T>* p1, const cplx<T>* p2, const cplx<T>* p3, size_t tot,
                         const double* __restrict__ w, const cplx<T>* pbc = nullptr,
                         const double* __restrict__ wbc = nullptr) {
  const double w1 = w[0], w2 = w[1], w3 = w[2];
  const double wb = pbc ? *wbc : 0.0;
  if constexpr (std::is_same<T, float>::value) {
    // FP32 grids: the weighted sum as a float pair, ~48 bits before the final
    // rounding, on the FP32 pipes (the FP64 rate bounded this pass)
    float wh[4], wl[4];
    const double wd[4] = {w1, w2, w3, wb};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      wh[q] = __double2float_rn(wd[q]);
      wl[q] = __double2float_rn(wd[q] - (double)wh[q]);
    }
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
      const float2 a = p1[idx];
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
      ff_axpy(wh[0], wl[0], a.x, rh, rl);
      ff_axpy(wh[0], wl[0], a.y, ih, il);
      if (p2) { const float2 b = p2[idx]; ff_axpy(wh[1], wl[1], b.x, rh, rl); ff_axpy(wh[1], wl[1], b.y, ih, il); }
      if (p3) { const float2 c = p3[idx]; ff_axpy(wh[2], wl[2], c.x, rh, rl); ff_axpy(wh[2], wl[2], c.y, ih, il); }
      if (pbc) { const float2 b = pbc[idx]; ff_axpy(wh[3], wl[3], b.x, rh, rl); ff_axpy(wh[3], wl[3], b.y, ih, il); }
      out[idx] = make_float2(rh + rl, ih + il);
    }
    return;
  }
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const cplx<T> a = p1[idx];
    double r = w1 * (double)a.x, im = w1 * (double)a.y;
    if (p2) { const cplx<T> b = p2[idx]; r += w2 * (double)b.x; im += w2 * (double)b.y; }
    if (p3) { const cplx<T> c = p3[idx]; r += w3 * (double)c.x; im += w3 * (double)c.y; }
    // the relative-velocity term of a two-species run (ic_generator.cc:907-910)
    if (pbc) { const cplx<T> b = pbc[idx]; r += wb * (double)b.x; im += wb * (double)b.y; }
    out[idx] = mkc<T>(T(r), T(im));
  }
}

// lattice readout of the three components of one sub-lattice
// (set_positions / set_velocities, particle_generator.hh:499-639): particle
// ip = ishift*n^3 + cell, AoS [ip][3]; positions q + Psi in FP64 with
// q_d = (idx_d + s_d)/n * lunit (get_unit_r_shifted, grid_fft.hh:242-252)
template <typename T, typename P>
__global__ void k_lattice3(const T* psi0, const T* psi1, const T* psi2, int n, P* dst, int ishift,
                           const double* __restrict__ q, int with_q, int fields_mode,
                           const float2* __restrict__ qf = nullptr) {
  const size_t n3 = (size_t)n * n * n;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n3; c += (size_t)gridDim.x * blockDim.x) {
    const size_t line = c / n;
    const int k = (int)(c % n);
    const size_t off = line * (n + 2) + k;
    if constexpr (std::is_same<P, float>::value && std::is_same<T, float>::value) {
      if (with_q && !fields_mode) {  // FP32 positions: q as a float pair (ff_add_q)
        const int j = (int)(line % n), i = (int)(line / n);
        P* o = dst + 3 * ((size_t)ishift * n3 + c);
        o[0] = ff_add_q(qf[i], psi0[off]);
        o[1] = ff_add_q(qf[n + j], psi1[off]);
        o[2] = ff_add_q(qf[2 * n + k], psi2[off]);
        continue;
      }
    }
    double v0 = (double)psi0[off], v1 = (double)psi1[off], v2 = (double)psi2[off];
    if (fields_mode) {
      dst[c] = (P)v0;
      dst[n3 + c] = (P)v1;
      dst[2 * n3 + c] = (P)v2;
      continue;
    }
    if (with_q) {  // q_d = (idx_d + s_d) / n * lunit, tabulated on the host
      const int j = (int)(line % n), i = (int)(line / n);
      v0 = q[i] + v0;
      v1 = q[n + j] + v1;
      v2 = q[2 * n + k] + v2;
    }
    P* o = dst + 3 * ((size_t)ishift * n3 + c);
    o[0] = (P)v0;
    o[1] = (P)v1;
    o[2] = (P)v2;
  }
}

// PLT gradient and growth-rate correction of every N-grid mode, tabulated
// once per pipeline (they depend on the lattice, N and the PLT mesh only):
// out[4 idx + {0,1,2,3}] = g_x, g_y, g_z, vfac_corr
template <typename T>
__global__ void k_plt_grad_table(T* __restrict__ out, int n, PLTDev<T> P) {
  const int Kz = n / 2 + 1;
  const size_t tot = (size_t)n * n * Kz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % Kz);
    const int j = (int)((idx / Kz) % n);
    const int i = (int)(idx / ((size_t)Kz * n));
    T g[3], vc = T(1);
    plt_gradient<T>(P, i, j, kz, g, &vc);
    out[4 * idx + 0] = g[0];
    out[4 * idx + 1] = g[1];
    out[4 * idx + 2] = g[2];
    out[4 * idx + 3] = vc;
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
// shift of the secondary (baryon) lattice (particle_generator.hh:56-63)
const double kSecondShift[4][3] = {{0.5, 0.5, 0.5}, {0.5, 0.5, 0.0}, {0.5, 0.5, 0.5}, {0.25, 0.25, 0.25}};

// shift_field chain of sub-lattice ish (particle_generator.hh:389-401, :510-522,
// :607-618): the secondary lattice's global shift first, then the relative
// shifts of sub-lattices 1..ish, in quarter cells
template <typename T>
ShiftChain<T> lattice_chain(const void* phase, int lattice, bool secondary, int ish) {
  ShiftChain<T> ch{};
  ch.phase = (const cplx<T>*)phase;
  ch.nstep = 0;
  if (secondary) {
    for (int q = 0; q < 3; ++q) ch.s4[0][q] = (int)lround(4 * kSecondShift[lattice][q]);
    ch.nstep = 1;
  }
  for (int st = 1; st <= ish; ++st, ++ch.nstep)
    for (int q = 0; q < 3; ++q)
      ch.s4[ch.nstep][q] = (int)lround(4 * (kShifts[lattice][st][q] - kShifts[lattice][st - 1][q]));
  return ch;
}

// device table of lattice coordinates: the doubles q[ishift][d][idx],
// followed by the same values as float pairs (hi, lo) for FP32 positions
cudaError_t upload_lattice_table(const std::vector<double>& q, double** out) {
  std::vector<double> buf(2 * q.size());
  std::copy(q.begin(), q.end(), buf.begin());
  float2* qf = reinterpret_cast<float2*>(buf.data() + q.size());
  for (size_t i = 0; i < q.size(); ++i) {
    const float hi = (float)q[i];
    qf[i] = make_float2(hi, (float)(q[i] - (double)hi));
  }
  cudaError_t e = cudaMalloc(out, buf.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(*out, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice);
  return e;
}

}  // namespace
}  // namespace mf

using namespace mf;

struct mf_ic {
  mf_ctx* ctx = nullptr;
  mf_ic_params p{};
  mf_grid* wn = nullptr;
  mf_grid* f[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // phi, phi2, phi3, A3x, A3y, A3z
  mf_grid* tmp[3] = {nullptr, nullptr, nullptr};  // real-space components of one sub-lattice
  void* phase = nullptr;  // exp(+2 pi i m / 4n), m in [0, 4n), grid precision
  double* qtab = nullptr; // lattice coordinates q[ishift][d][idx] * lunit
  void* plt = nullptr;    // PLT tables Dr, Dth, Dph, Dvf in the grid precision
  void* pltg = nullptr;   // PLT gradient and vfac_corr per N-grid mode [idx][4]
  double* stage = nullptr;  // n^3 doubles: host noise upload of an FP32 pipeline
  int plt_ng = 0;
  mf_conv* conv = nullptr;
  double* amp = nullptr;
  int nk2 = 0;
  void* dpos = nullptr;
  void* dvel = nullptr;
  void* dids = nullptr;
  size_t pos_bytes = 0, vel_bytes = 0, id_bytes = 0;
  // two species: the baryons' particle arrays, both species' masses, the
  // baryon-CDM amplitude tables and fields
  void* bpos = nullptr;
  void* bvel = nullptr;
  void* bids = nullptr;
  void* dmass[2] = {nullptr, nullptr};
  size_t mass_bytes = 0;
  double* bqtab = nullptr;  // secondary-lattice coordinates, as qtab
  double* ampbc = nullptr;  // [0, nk2) amp_dbc, [nk2, 2 nk2) amp_tbc, then the host tables
  const double* tdbc_d = nullptr;
  const double* ttbc_d = nullptr;
  mf_grid* rho_bc = nullptr;  // k-space wn amp_dbc
  mf_grid* psi_bc = nullptr;  // k-space amp_tbc wn / k^2
  mf_grid* rho_e = nullptr;   // k-space wn amp_dbc without the relative-velocity mode (Eulerian branch)
  void* ppt = nullptr;        // Eulerian-branch scratch: two FP64 real grids, 3 n^3 complex, one scalar
  int64_t npart = 0;
  cudaEvent_t ev[9] = {};
  bool noise_set = false;   // an uploaded white-noise field is waiting in wn
  bool noise_seeded = false; // the device generator fills wn at the start of each run
  bool has_tk = false;      // amp + nk2 holds a tabulated T(k)
  ICDyn* dyn_h = nullptr;   // page-locked host copy, copied to dyn_d at the start of each run
  ICDyn* dyn_d = nullptr;
  // host hand-off: the particles are copied on a second stream while the
  // rest of the run computes.  ev_copy follows the last copy queued on it,
  // ev_ids the last copy of the IDs; a run waits for them before it writes
  // the particle buffers again, so an asynchronous run's copies overlap the
  // next run's fields
  cudaStream_t cstream = nullptr;
  cudaEvent_t ev_pos = nullptr, ev_copy = nullptr, ev_ids = nullptr;
  mf_particles early_out{};  // host destinations of the run being enqueued asynchronously
  // host noise uploads of an FP32 pipeline: copied into the staging buffer on
  // their own stream once the previous upload has been converted, so that an
  // upload overlaps the run before it
  cudaStream_t hstream = nullptr;
  cudaEvent_t ev_stage_free = nullptr, ev_stage_full = nullptr;
  const mf_particles* early = nullptr;
  bool early_all = false;  // every particle array was streamed to the host during the run
  bool pos_early = false;  // the positions were copied during the run
  bool ids_early = false;  // the IDs were copied during the run
  // shared-source convolutions: padded real fields and three work buffers
  bool shared = false;
  void* rf = nullptr;   // real padded fields [nreal][M*M][M/2] packed pairs (last 5 or 1: product sums)
  void* w3 = nullptr;   // three work buffers [M][M][N/2+1] complex
};

namespace {

// the Orszag source terms through shared padded real fields (default), or
// one convolution per term (per_term_conv, or the aliased convolver)
bool uses_shared_sources(const mf_ic_params* p) {
  return p->lpt_order > 1 && p->convolver == MF_CONV_ORSZAG && !p->per_term_conv;
}

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
  if (p->plt && p->plt_ngrid != 0 && !grid_size_supported(p->plt_ngrid)) return MF_ERR_SHAPE;
  if (p->baryons) {
    if (!(p->munit > 0) || !(p->cosmo.Omega_b > 0) || !(p->cosmo.Omega_m > p->cosmo.Omega_b)) return MF_ERR_ARG;
    if (p->Dplus_target < 0) return MF_ERR_ARG;
  }
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

// growth-factor weights of the two assembly passes (ic_generator.cc:221-234,
// :835-845, :889-899): positions g_n, velocities n vfac g_n; the A3 term
// carries g3c = D^3/7 (times 3 vfac for velocities)
void fill_dyn(mf_ic* ic) {
  const mf_ic_params& p = ic->p;
  ICDyn& d = *ic->dyn_h;
  eh_setup(p.cosmo.H0 > 0 ? p.cosmo.H0 : 100.0 * p.cosmo.h, p.cosmo.Omega_m, p.cosmo.Omega_b, p.cosmo.Tcmb, &d.eh);
  d.half_ns = 0.5 * p.cosmo.n_s;
  d.sqrtpnorm = std::sqrt(p.cosmo.pnorm);
  const double D = p.cosmo.Dplus, vf = p.cosmo.vfac;
  const double g1 = -D;
  const double g2 = (p.lpt_order > 1) ? -3.0 / 7.0 * D * D : 0.0;
  const double g3 = (p.lpt_order > 2) ? 1.0 / 3.0 * D * D * D : 0.0;
  const double g3c = (p.lpt_order > 2) ? 1.0 / 7.0 * D * D * D : 0.0;
  d.w[0][0] = g1; d.w[0][1] = g2; d.w[0][2] = g3; d.w[0][3] = g3c;
  d.w[1][0] = vf * g1; d.w[1][1] = 2 * vf * g2; d.w[1][2] = 3 * vf * g3; d.w[1][3] = 3 * vf * g3c;
  if (p.baryons) {
    const double Om = p.cosmo.Omega_m, Ob = p.cosmo.Omega_b, fb = Ob / Om;
    d.Cs[0] = -fb;        // dark matter
    d.Cs[1] = 1.0 - fb;   // baryons
    d.Omega_s[0] = Om - Ob;
    d.Omega_s[1] = Ob;
    d.vrel = p.baryon_vrel ? 1 : 0;
    d.wbc[0] = d.vrel ? -vf * d.Cs[0] : 0.0;
    d.wbc[1] = d.vrel ? -vf * d.Cs[1] : 0.0;
    d.bc_Dt = p.Dplus_target > 0 ? p.Dplus_target : 1.0;
    d.bc_sqrtDr = std::sqrt(d.bc_Dt / D);
  }
}

// phi(2), phi(3) and A(3) with shared padded real fields (ic_generator.cc:471-545).
// Every Orszag convolution of the reference multiplies two padded operands in
// real space, transforms the product back and unpads it into the target
// through a linear op::.  By linearity of the r2c and of the unpad, the sum
// of the target's convolutions equals one r2c and unpad of the sum of the
// real-space products, so each distinct operand (the six Hessians of phi,
// the six of phi(2), the five truncated pair products of convolve3's first
// stage) is transformed to padded real space once, and each target is one
// product sum, one r2c and one unpad.  convolve3 keeps its intermediate
// truncation: the pair product is unpadded into an N-grid (Nyquist zeroed)
// and transformed again before the third factor multiplies it.
template <typename T>
int shared_sources(mf_ic* ic, bool timed) {
  mf_ctx* c = ic->ctx;
  cudaStream_t s = c->stream;
  const mf_ic_params& p = ic->p;
  const int N = p.ngrid, M = 3 * N / 2, Kz = N / 2 + 1, H = M / 2;
  const ConvGeom g{N, M, Kz, true};
  const T kfac = T(2.0 * M_PI / p.boxlen);
  const double M3 = (double)M * M * M, N3 = (double)N * N * N;
  const T scale_in = T(std::pow(1.5, 1.5) / std::sqrt(M3));
  const T scale_out = T(1.0 / std::sqrt(M3) / (std::sqrt(M3) / std::sqrt(N3)));
  const cplx<T>* twM = c->tw.get<T>(M, s);
  const cplx<T>* twH = c->tw.get<T>(H, s);
  if (!twM || !twH) return set_err(c, MF_ERR_OOM, "twiddles");
  const size_t per = (size_t)M * M * Kz;
  cplx<T>* W[3] = {(cplx<T>*)ic->w3, (cplx<T>*)ic->w3 + per, (cplx<T>*)ic->w3 + 2 * per};
  const size_t rl = (size_t)M * M * H;
  auto R = [&](int i) { return (cplx<T>*)ic->rf + (size_t)i * rl; };
  cudaError_t e;
#define CK(x)                                            \
  do {                                                   \
    e = (x);                                             \
    if (e != cudaSuccess) return cuda_err(c, e, #x);     \
  } while (0)

  // padded c2r of up to three operands into real fields dst[k]
  auto c2r = [&](int nop, const Operand<T>* ops, const int* dst) -> cudaError_t {
    ConvXInvOp<T> xo{};
    for (int k = 0; k < nop; ++k) { xo.opnd[k] = ops[k]; xo.dst[k] = W[k]; }
    xo.g = g;
    xo.kfac = kfac;
    xo.scale = scale_in;
    cudaError_t e2;
    {
      LaunchScope ls(c, KK_CONV_XINV);
      if ((e2 = Launch<T>::conv_xinv(M, xo, N, Kz, nop, twM, s)) != cudaSuccess) return e2;
    }
    ConvYInvOp<T> yo{};
    for (int k = 0; k < nop; ++k) { yo.src[k] = W[k]; yo.dst[k] = W[k]; }
    yo.g = g;
    {
      LaunchScope ls(c, KK_CONV_YINV);
      if ((e2 = Launch<T>::conv_yinv(M, yo, M, Kz, nop, twM, s)) != cudaSuccess) return e2;
    }
    for (int k = 0; k < nop; ++k) {
      ZConvArgs<T> za{};
      za.in[0] = W[k];
      za.out = R(dst[k]);
      za.nop = 1;
      za.kin = Kz;
      za.kout = H;
      za.in_stride = Kz;
      za.out_stride = H;
      za.nlines = M * M;
      za.out_scale = T(1);
      za.err = c->d_err;
      LaunchScope ls(c, KK_CONV_Z);
      if ((e2 = Launch<T>::z_c2r_tma(H, za, twH, twM, s)) != cudaSuccess) return e2;
    }
    return cudaSuccess;
  };
  // product-sum scratch fields (after the 17 operand fields)
  const int P0 = (p.lpt_order > 2) ? 17 : 6;
  // TMA r2c of real field `src`, unpadded into target with op:: (and -1/k^2)
  auto r2c_unpad = [&](int src, cplx<T>* target, int op, int invlap) -> cudaError_t {
    ZConvArgs<T> za{};
    za.in[0] = R(src);
    za.out = W[0];
    za.nop = 1;
    za.kin = H;
    za.kout = Kz;
    za.in_stride = H;
    za.out_stride = Kz;
    za.nlines = M * M;
    za.out_scale = T(1);
    za.err = c->d_err;
    cudaError_t e2;
    {
      LaunchScope ls(c, KK_CONV_Z);
      if ((e2 = Launch<T>::z_r2c_tma(H, za, twH, twM, s)) != cudaSuccess) return e2;
    }
    ConvYFwdOp<T> yf{W[0], W[0], g};
    {
      LaunchScope ls(c, KK_CONV_YFWD);
      if ((e2 = Launch<T>::conv_yfwd(M, yf, M, Kz, twM, s)) != cudaSuccess) return e2;
    }
    ConvXFwdOp<T> xf{};
    xf.src = W[0];
    xf.target = target;
    xf.g = g;
    xf.scale = scale_out;
    xf.out_op = op;
    xf.x = T(1);
    xf.post_invlap = invlap;
    xf.kfac = kfac;
    LaunchScope ls(c, KK_CONV_XFWD);
    return Launch<T>::conv_xfwd(M, xf, N, Kz, twM, s);
  };
  // the streaming product kernel of one source set (mf_sources.cu) into P0, P0+1, ...
  auto sources = [&](int set) -> cudaError_t {
    const T* fields[kSrcFields] = {};
    for (int f = 0; f < kSrcFields; ++f)
      if (f < P0) fields[f] = (const T*)R(f);
    T* outs[kSrcOutputs] = {};
    for (int o = 0; o < kSrcOutputs; ++o)
      if (P0 + o < ((p.lpt_order > 2) ? 22 : 7)) outs[o] = (T*)R(P0 + o);
    if (set == SRC_PHI2_PAIRS)  // the pairs go to the (still unused) slots of the phi(2) Hessians
      for (int o = 1; o < 6; ++o) outs[o] = (T*)R(5 + o);
    LaunchScope ls(c, KK_POINTWISE);
    return pw_sources<T>(set, fields, outs, 2 * rl, s);
  };
  // Hessian fields in the order (0,0) (1,1) (2,2) (0,1) (0,2) (1,2)
  const int HD[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  auto hessians = [&](int fi, int base) -> cudaError_t {
    for (int half = 0; half < 2; ++half) {
      Operand<T> ops[3];
      int dst[3];
      for (int k = 0; k < 3; ++k) {
        ops[k] = Operand<T>{};
        ops[k].f = (const cplx<T>*)ic->f[fi]->d;
        ops[k].kind = OPND_HESS;
        ops[k].d[0] = HD[3 * half + k][0];
        ops[k].d[1] = HD[3 * half + k][1];
        dst[k] = base + 3 * half + k;
      }
      cudaError_t e2 = c2r(3, ops, dst);
      if (e2 != cudaSuccess) return e2;
    }
    return cudaSuccess;
  };

  // convolve3's first stage for one pair product held as a padded real field:
  // r2c, the truncation to the N-cube (unpad with the Nyquist planes zeroed,
  // convolution.hh:543-549, :618-653) and the padded c2r of the truncated
  // field (pad_insert, :570-592) into another real field.  The x passes of
  // the two transforms and the truncation are one pass (ConvXTruncOp), so the
  // unpadded N-grid never goes to HBM.
  auto truncate_pair = [&](int src, int dstf) -> cudaError_t {
    cudaError_t e2;
    ZConvArgs<T> za{};
    za.in[0] = R(src);
    za.out = W[0];
    za.nop = 1;
    za.kin = H;
    za.kout = Kz;
    za.in_stride = H;
    za.out_stride = Kz;
    za.nlines = M * M;
    za.out_scale = T(1);
    za.err = c->d_err;
    {
      LaunchScope ls(c, KK_CONV_Z);
      if ((e2 = Launch<T>::z_r2c_tma(H, za, twH, twM, s)) != cudaSuccess) return e2;
    }
    ConvYFwdOp<T> yf{W[0], W[0], g};
    {
      LaunchScope ls(c, KK_CONV_YFWD);
      if ((e2 = Launch<T>::conv_yfwd(M, yf, M, Kz, twM, s)) != cudaSuccess) return e2;
    }
    ConvXTruncOp<T> xt{W[0], g, scale_out, scale_in};
    {
      LaunchScope ls(c, KK_CONV_XFWD);
      if ((e2 = Launch<T>::conv_xtrunc(M, xt, N, Kz, twM, s)) != cudaSuccess) return e2;
    }
    ConvYInvOp<T> yo{};
    yo.src[0] = W[0];
    yo.dst[0] = W[0];
    yo.g = g;
    {
      LaunchScope ls(c, KK_CONV_YINV);
      if ((e2 = Launch<T>::conv_yinv(M, yo, M, Kz, 1, twM, s)) != cudaSuccess) return e2;
    }
    ZConvArgs<T> zc{};
    zc.in[0] = W[0];
    zc.out = R(dstf);
    zc.nop = 1;
    zc.kin = Kz;
    zc.kout = H;
    zc.in_stride = Kz;
    zc.out_stride = H;
    zc.nlines = M * M;
    zc.out_scale = T(1);
    zc.err = c->d_err;
    LaunchScope ls(c, KK_CONV_Z);
    return Launch<T>::z_c2r_tma(H, zc, twH, twM, s);
  };

  // ---- phi(2) (ic_generator.cc:471-488) ----------------------------------
  // with 3LPT the convolve3 first stages (truncated pair products phi,00 phi,11
  // / phi,01 phi,02 / phi,12^2 / phi,02^2 / phi,01^2) come out of the same pass
  CK(hessians(0, 0));
  CK(sources(p.lpt_order > 2 ? SRC_PHI2_PAIRS : SRC_PHI2));
  CK(r2c_unpad(P0, (cplx<T>*)ic->f[1]->d, OUT_ASSIGN, 1));
  ic->f[1]->space = MF_SPACE_K;
  // the truncated pairs, from the slots of the phi(2) Hessians (still free)
  // into their operand slots 12..16
  if (p.lpt_order > 2)
    for (int k = 0; k < 5; ++k) CK(truncate_pair(6 + k, 12 + k));
  if (timed) CK(cudaEventRecord(ic->ev[2], s));
  if (p.lpt_order > 2) {
    // ---- phi(3) (ic_generator.cc:511-528) --------------------------------
    CK(hessians(1, 6));
    CK(sources(SRC_PHI3_A3));
    CK(r2c_unpad(P0, (cplx<T>*)ic->f[2]->d, OUT_ASSIGN, 1));
    ic->f[2]->space = MF_SPACE_K;
    if (timed) CK(cudaEventRecord(ic->ev[3], s));
    // ---- A(3) (ic_generator.cc:534-545) ---------------------------------
    for (int d = 0; d < 3; ++d) {
      CK(r2c_unpad(P0 + 1 + d, (cplx<T>*)ic->f[3 + d]->d, OUT_ASSIGN, 1));
      ic->f[3 + d]->space = MF_SPACE_K;
    }
  } else if (timed) {
    CK(cudaEventRecord(ic->ev[3], s));
  }
#undef CK
  return MF_OK;
}

// the whole pipeline on the context's stream, without host synchronisation
// or host-side data dependencies: safe to record into a CUDA graph once the
// twiddle tables exist (mf_ic_create builds them)
template <typename T>
int enqueue_impl(mf_ic* ic) {
  mf_ctx* c = ic->ctx;
  cudaStream_t s = c->stream;
  const mf_ic_params& p = ic->p;
  const int n = p.ngrid, Kz = n / 2 + 1;
  const double L = p.boxlen, kfac = 2.0 * M_PI / L;
  const size_t nk = (size_t)n * n * Kz;
  const bool timed = !c->capturing;
  cudaError_t e;
#define CK(x)                                            \
  do {                                                   \
    e = (x);                                             \
    if (e != cudaSuccess) return cuda_err(c, e, #x);     \
  } while (0)

  if (timed) CK(cudaEventRecord(ic->ev[0], s));
  CK(cudaMemcpyAsync(ic->dyn_d, ic->dyn_h, sizeof(ICDyn), cudaMemcpyHostToDevice, s));
  const bool fields = p.out_kind == MF_OUT_FIELDS;
  const int overload = 1 << p.lattice;
  // host hand-off during the run: each particle array (or sub-lattice slice)
  // is copied on the copy stream as soon as it is final
  auto early_copy = [&](void* hdst, const void* dsrc, size_t bytes) -> cudaError_t {
    cudaError_t e2 = cudaEventRecord(ic->ev_pos, s);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(ic->cstream, ic->ev_pos, 0);
    if (e2 == cudaSuccess) e2 = cudaMemcpyAsync(hdst, dsrc, bytes, cudaMemcpyDeviceToHost, ic->cstream);
    if (e2 == cudaSuccess) e2 = cudaEventRecord(ic->ev_copy, ic->cstream);
    return e2;
  };
  // ---- particle IDs (particle_generator.hh:212-253): independent of the
  // fields, so they are made first and their copy overlaps the whole run
  if (!fields) {
    // (after the previous run's copy of them, which may still be queued)
    if (!c->capturing && ic->ev_ids) CK(cudaStreamWaitEvent(s, ic->ev_ids, 0));
    LaunchScope ls(c, KK_POINTWISE);
    if (p.id64)
      k_ids<uint64_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint64_t*)ic->dids, n, overload, 0);
    else
      k_ids<uint32_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint32_t*)ic->dids, n, overload, 0);
    CK(cudaGetLastError());
    if (ic->early) {  // the IDs' copy overlaps the whole run
      CK(early_copy(ic->early->ids, ic->dids, ic->id_bytes));
      CK(cudaEventRecord(ic->ev_ids, ic->cstream));
      ic->ids_early = true;
    }
    if (p.baryons) {  // baryon IDs start at IDoffset = 1 (ic_generator.cc:626-628)
      const uint64_t off = (uint64_t)overload * n * n * n;
      if (p.id64)
        k_ids<uint64_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint64_t*)ic->bids, n, overload, off);
      else
        k_ids<uint32_t><<<blocks_for((size_t)n * n * n), kThreads, 0, s>>>((uint32_t*)ic->bids, n, overload, off);
      CK(cudaGetLastError());
    }
  }
  // ---- white noise (RNG_plugin::Fill_Grid) to k-space, phi(1) -----------------
  if (ic->noise_seeded) {
    LaunchScope ls(c, KK_POINTWISE);
    CK(pw_white_noise<T>((T*)ic->wn->d, n, 0ull, &ic->dyn_d->seed, s));
  }
  CK(fft3d_r2c<T>(c, (T*)ic->wn->d, n));
  ic->wn->space = MF_SPACE_K;
  {
    LaunchScope ls0(c, KK_POINTWISE);
    k_amp_table<<<(ic->nk2 + 255) / 256, 256, 0, s>>>(ic->amp, ic->nk2, kfac, ic->dyn_d,
                                                       ic->has_tk ? ic->amp + ic->nk2 : nullptr);
    CK(cudaGetLastError());
    const double volfac = std::pow(L / n / 2.0 / M_PI, 1.5);
    const double sgn = (p.inversion ? -1.0 : 1.0) / volfac;
    LaunchScope ls1(c, KK_POINTWISE);
    k_phi1<T><<<blocks_for(nk), kThreads, 0, s>>>((cplx<T>*)ic->wn->d, (cplx<T>*)ic->f[0]->d, n, kfac, ic->amp, sgn,
                                                   p.fixing);
    CK(cudaGetLastError());
    ic->f[0]->space = MF_SPACE_K;
  }
  // ---- baryon-CDM fields of a two-species run, from the normalised noise
  // before its grid is reused (ic_generator.cc:655-660, :907-910)
  if (ic->rho_bc) {
    LaunchScope ls(c, KK_POINTWISE);
    double* ampd = ic->ampbc;
    double* ampt = ic->ampbc + ic->nk2;
    double* ampd0 = ic->ampbc + 2 * ic->nk2;
    k_amp_bc<<<(ic->nk2 + 255) / 256, 256, 0, s>>>(ampd, ampt, ampd0, ic->nk2, kfac, ic->dyn_d, ic->tdbc_d,
                                                   ic->ttbc_d);
    CK(cudaGetLastError());
    k_bc_fields<T><<<blocks_for(nk), kThreads, 0, s>>>(
        (const cplx<T>*)ic->wn->d, (cplx<T>*)ic->rho_bc->d, ic->psi_bc ? (cplx<T>*)ic->psi_bc->d : nullptr,
        ic->rho_e ? (cplx<T>*)ic->rho_e->d : nullptr, n, kfac, ampd, ampt, ampd0);
    CK(cudaGetLastError());
  }
  if (timed) CK(cudaEventRecord(ic->ev[1], s));

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

  if (ic->shared) {
    const int rc = shared_sources<T>(ic, timed);
    if (rc != MF_OK) return rc;
  }
  // ---- phi(2) (ic_generator.cc:471-488) ----------------------------------
  if (p.lpt_order > 1 && !ic->shared) {
    CK(conv2(H(0, 0, 0), S(0, 1, 1, 2, 2, false), 1, OUT_ASSIGN, 1, 0));
    CK(conv2(H(0, 1, 1), H(0, 2, 2), 1, OUT_ADD, 1, 0));
    CK(conv2(H(0, 0, 1), H(0, 0, 1), 1, OUT_SUB, 1, 0));
    CK(conv2(H(0, 0, 2), H(0, 0, 2), 1, OUT_SUB, 1, 0));
    CK(conv2(H(0, 1, 2), H(0, 1, 2), 1, OUT_SUB, 1, 1));
    ic->f[1]->space = MF_SPACE_K;
  }
  if (timed && !ic->shared) CK(cudaEventRecord(ic->ev[2], s));
  // ---- phi(3) (ic_generator.cc:511-528) ----------------------------------
  if (p.lpt_order > 2 && !ic->shared) {
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
  if (timed && !ic->shared) CK(cudaEventRecord(ic->ev[3], s));
  // ---- A(3) (ic_generator.cc:534-545) -----------------------------------
  if (p.lpt_order > 2 && !ic->shared) {
    for (int d = 0; d < 3; ++d) {
      const int dp = (d + 1) % 3, dpp = (d + 2) % 3, tg = 3 + d;
      CK(conv2(H(1, d, dp), H(0, d, dpp), tg, OUT_ASSIGN, 1, 0));
      CK(conv2(H(1, d, dpp), H(0, d, dp), tg, OUT_SUB, 1, 0));
      CK(conv2(H(0, dp, dpp), S(1, dp, dp, dpp, dpp, true), tg, OUT_ADD, 1, 0));
      CK(conv2(H(1, dp, dpp), S(0, dp, dp, dpp, dpp, true), tg, OUT_SUB, 1, 1));
      ic->f[tg]->space = MF_SPACE_K;
    }
  }
  if (timed) CK(cudaEventRecord(ic->ev[4], s));

  T* wsum = (T*)ic->wn->d;  // the noise grid is free after phi(1): holds the order sum
  const cplx<T>* P1 = (const cplx<T>*)ic->f[0]->d;
  const cplx<T>* P2 = ic->f[1] ? (const cplx<T>*)ic->f[1]->d : nullptr;
  const cplx<T>* P3 = ic->f[2] ? (const cplx<T>*)ic->f[2]->d : nullptr;
  const cplx<T>* twN = c->tw.get<T>(n, s);
  const cplx<T>* twH = c->tw.get<T>(n / 2, s);
  if (!twN || !twH) return set_err(c, MF_ERR_OOM, "twiddles");
  const size_t n3 = (size_t)n * n * n;
  // species of the Lagrangian assembly: dark matter, then the baryons on the
  // secondary lattice; with field output the baryons take the Eulerian branch
  const int nsp = (p.baryons && !fields) ? 2 : 1;
  // the particle buffers are rewritten below: after every copy of them that
  // an earlier asynchronous run queued on the copy stream
  if (!c->capturing && ic->ev_copy) CK(cudaStreamWaitEvent(s, ic->ev_copy, 0));
  for (int pass = 0; pass < 2; ++pass) {  // 0: positions, 1: velocities
    const bool vel = pass == 1;
    for (int sp = 0; sp < nsp; ++sp) {
    // the order sum is the same for both species unless the velocities carry
    // the species' relative-velocity term
    const bool bc_term = vel && ic->psi_bc;
    if (sp == 0 || bc_term) {
      LaunchScope ls(c, KK_POINTWISE);
      k_phitot<T><<<blocks_for(nk), kThreads, 0, s>>>(
          (cplx<T>*)wsum, P1, p.lpt_order > 1 ? P2 : nullptr, p.lpt_order > 2 ? P3 : nullptr, nk, ic->dyn_d->w[pass],
          bc_term ? (const cplx<T>*)ic->psi_bc->d : nullptr, &ic->dyn_d->wbc[sp]);
      CK(cudaGetLastError());
    }
    void* dst = sp ? (vel ? ic->bvel : ic->bpos) : (vel ? ic->dvel : ic->dpos);
    const double* qbase = sp ? ic->bqtab : ic->qtab;
    const float2* qfbase = reinterpret_cast<const float2*>(qbase + (size_t)overload * 3 * n);
    const bool three = Launch<T>::assemble3_supported(n);
    for (int ish = 0; ish < overload; ++ish) {
      if (three) {  // x pass of the three components in one launch
        Assemble3XInvOp<T> op{};
        op.phitot = (const cplx<T>*)wsum;
        for (int d = 0; d < 3; ++d) {
          op.A3[d] = p.lpt_order > 2 ? (const cplx<T>*)ic->f[3 + d]->d : nullptr;
          op.dst[d] = (cplx<T>*)ic->tmp[d]->d;
        }
        op.n = n;
        op.Kz = Kz;
        op.ch = lattice_chain<T>(ic->phase, p.lattice, sp == 1, ish);
        op.kfac = T(kfac);
        op.wA = &ic->dyn_d->w[pass][3];
        op.unit = T((vel ? p.vunit : p.lunit) / L);
        op.plt = p.plt;
        op.vel = vel ? 1 : 0;
        op.pg = (const T*)ic->pltg;
        LaunchScope ls(c, KK_FFT_COL);
        CK(Launch<T>::assemble3_xinv(n, op, n, Kz, twN, s));
      }
      for (int d = 0; d < 3; ++d) {
        T* tmpr = (T*)ic->tmp[d]->d;
        cplx<T>* tk = (cplx<T>*)tmpr;
        AssembleXInvOp<T> op{};
        op.phitot = (const cplx<T>*)wsum;
        op.A3p = p.lpt_order > 2 ? (const cplx<T>*)ic->f[3 + (d + 1) % 3]->d : nullptr;
        op.A3pp = p.lpt_order > 2 ? (const cplx<T>*)ic->f[3 + (d + 2) % 3]->d : nullptr;
        op.dst = tk;
        op.n = n;
        op.Kz = Kz;
        op.d = d;
        op.ch = lattice_chain<T>(ic->phase, p.lattice, sp == 1, ish);
        op.kfac = T(kfac);
        op.wA = &ic->dyn_d->w[pass][3];
        op.unit = T((vel ? p.vunit : p.lunit) / L);
        op.plt = p.plt;
        op.vel = vel ? 1 : 0;
        if (p.plt) {
          const size_t nkt = (size_t)ic->plt_ng * ic->plt_ng * (ic->plt_ng / 2 + 1);
          const T* base = (const T*)ic->plt;
          op.P.Dr = base;
          op.P.Dth = base + nkt;
          op.P.Dph = base + 2 * nkt;
          op.P.Dvf = base + 3 * nkt;
          op.P.ng = ic->plt_ng;
          op.P.mapratio = T((double)ic->plt_ng / (double)n);
          op.P.inv_mr_L = T(1.0 / ((double)ic->plt_ng / (double)n) / L);
          op.pg = (const T*)ic->pltg;
        }
        if (!three) {
          LaunchScope ls(c, KK_FFT_COL);
          CK(Launch<T>::assemble_xinv(n, op, n, Kz, twN, s));
        }
        {
          LaunchScope ls(c, KK_FFT_COL);
          CK(Launch<T>::colfft_plain(n, true, PlainStridedOp<T>{tk, Kz, (long long)n * Kz, T(1)}, n, Kz, twN, s));
        }
        if (!three) {
          LaunchScope ls(c, KK_FFT_Z);
          const T norm = T(1.0 / std::sqrt((double)n * (double)n * (double)n));
          CK(Launch<T>::z_c2r_plain(n / 2, PlainZOp<T>{tmpr, n, norm}, n * n, Kz, twH, twN, s));
        }
      }
      const double* qt = qbase + (size_t)ish * 3 * n;
      if (three) {  // the three components' z passes with the lattice readout fused
        Lattice3Args la{};
        for (int d = 0; d < 3; ++d) la.comp[d] = ic->tmp[d]->d;
        la.dst = dst;
        la.q = qt;
        la.qf = qfbase + (size_t)ish * 3 * n;
        la.n = n;
        la.nlines = n * n;
        la.ishift = fields ? 0 : ish;
        la.with_q = (!fields && !vel) ? 1 : 0;
        la.fields_mode = fields ? 1 : 0;
        la.norm = 1.0 / std::sqrt((double)n * (double)n * (double)n);
        {
          LaunchScope ls(c, KK_FFT_Z);
          CK(Launch<T>::z_c2r3_lattice(n / 2, la, fields || p.pos64, twH, twN, s));
        }
        if (ic->early && !fields && MF_STREAM_HANDOFF) {
          const size_t slice = (vel ? ic->vel_bytes : ic->pos_bytes) / overload;
          CK(early_copy((char*)(vel ? ic->early->vel : ic->early->pos) + ish * slice, (const char*)dst + ish * slice,
                        slice));
        }
        continue;
      }
      const T* q0 = (const T*)ic->tmp[0]->d;
      const T* q1 = (const T*)ic->tmp[1]->d;
      const T* q2 = (const T*)ic->tmp[2]->d;
      LaunchScope ls(c, KK_POINTWISE);
      if (fields)
        k_lattice3<T, double><<<blocks_for(n3), kThreads, 0, s>>>(q0, q1, q2, n, (double*)dst, 0, qt, 0, 1);
      else if (p.pos64)
        k_lattice3<T, double><<<blocks_for(n3), kThreads, 0, s>>>(q0, q1, q2, n, (double*)dst, ish, qt, vel ? 0 : 1, 0);
      else
        k_lattice3<T, float><<<blocks_for(n3), kThreads, 0, s>>>(q0, q1, q2, n, (float*)dst, ish, qt, vel ? 0 : 1, 0,
                                                                 qfbase + (size_t)ish * 3 * n);
      CK(cudaGetLastError());
      if (ic->early && !fields && MF_STREAM_HANDOFF) {
        const size_t slice = (vel ? ic->vel_bytes : ic->pos_bytes) / overload;
        CK(early_copy((char*)(vel ? ic->early->vel : ic->early->pos) + ish * slice, (const char*)dst + ish * slice,
                      slice));
      }
    }
    }  // species
    void* dst = vel ? ic->dvel : ic->dpos;
    if (timed) CK(cudaEventRecord(ic->ev[5 + pass], s));
    if (ic->early && (fields || !MF_STREAM_HANDOFF) && !vel)  // positions final: copy them during the velocity pass
      CK(early_copy(ic->early->pos, dst, ic->pos_bytes));
    if (ic->early && fields && MF_STREAM_HANDOFF && vel) CK(early_copy(ic->early->vel, dst, ic->vel_bytes));
  }
  // ---- particle masses of a two-species run (ic_generator.cc:641-673): per
  // particle, or the dark matter's mass field for field output ---------------
  if (p.baryons) {
    // set_masses with munit 1 (particle_generator.hh:383); a field is written as is
    const double pmean = fields ? 1.0 : 1.0 / ((double)n3 * overload);
    for (int sp = 0; sp < (fields ? 1 : 2); ++sp)
      for (int ish = 0; ish < overload; ++ish) {
        const T* delta = nullptr;
        if (ic->rho_bc) {
          cplx<T>* tk = (cplx<T>*)ic->tmp[0]->d;
          {
            LaunchScope ls(c, KK_POINTWISE);
            k_shift_chain<T><<<blocks_for(nk), kThreads, 0, s>>>((const cplx<T>*)ic->rho_bc->d, tk, n,
                                                                 lattice_chain<T>(ic->phase, p.lattice, sp == 1, ish));
            CK(cudaGetLastError());
          }
          CK(fft3d_c2r<T>(c, (T*)tk, n));
          delta = (const T*)tk;
        }
        LaunchScope ls(c, KK_POINTWISE);
        if (p.pos64 || fields)
          k_masses<T, double><<<blocks_for(n3), kThreads, 0, s>>>((double*)ic->dmass[sp], delta, n, ish, pmean, p.munit,
                                                                  ic->dyn_d, sp);
        else
          k_masses<T, float><<<blocks_for(n3), kThreads, 0, s>>>((float*)ic->dmass[sp], delta, n, ish, pmean, p.munit,
                                                                 ic->dyn_d, sp);
        CK(cudaGetLastError());
      }
  }
  // ---- baryons of a two-species field output: the semiclassical Eulerian
  // branch (ic_generator.cc:679-791) --------------------------------------------
  if (p.baryons && fields) {
    PPTArgs a{};
    a.n = n;
    a.L = L;
    a.f0 = ic->f[0]->d;
    a.f1 = p.lpt_order > 1 ? ic->f[1]->d : nullptr;
    a.g1 = ic->dyn_h->w[0][0];
    a.g2 = ic->dyn_h->w[0][1];
    mf_grid* de = ic->rho_e ? ic->rho_e : ic->rho_bc;
    a.delta_k = de ? de->d : nullptr;
    a.delta_r = ic->tmp[1]->d;
    a.C = ic->dyn_h->Cs[1];
    a.D = p.cosmo.Dplus;
    a.vunit = p.cosmo.Dplus * p.cosmo.vfac / L * p.vunit;
    char* b = (char*)ic->ppt;
    a.phi_r = (double*)b;
    a.phi2_r = a.phi_r + grid_reals(n);
    a.psi = (double2*)(a.phi2_r + grid_reals(n));
    a.grad = a.psi + n3;
    a.maxd = (double*)(a.grad + 2 * n3);
    a.rho_out = (double*)ic->bpos;
    a.vel_out = (double*)ic->bvel;
    CK((p.precision == MF_PREC_F64) ? ppt_eulerian<double>(c, a) : ppt_eulerian<float>(c, a));
  }
  if (timed) CK(cudaEventRecord(ic->ev[7], s));  // (the IDs are made at the start)
  if (ic->early) ic->early_all = MF_STREAM_HANDOFF;
  if (ic->early) ic->pos_early = true;
#undef CK
  return MF_OK;
}

// hand-off of the particles (device pointers, or copies into host buffers).
// Asynchronous (host buffers only): the copies not streamed during the run go
// on the copy stream too, and the context's stream does not wait for them
int handoff(mf_ic* ic, mf_particles* out, bool async) {
  mf_ctx* c = ic->ctx;
  cudaStream_t s = c->stream;
  const bool fields = ic->p.out_kind == MF_OUT_FIELDS;
  cudaError_t e;
#define CK(x)                                            \
  do {                                                   \
    e = (x);                                             \
    if (e != cudaSuccess) return cuda_err(c, e, #x);     \
  } while (0)
  if (out) {
    out->npart = ic->npart;
    if (out->location == MF_LOC_HOST) {
      if (!out->pos || !out->vel || (!fields && !out->ids)) return set_err(c, MF_ERR_ARG, "mf_ic_run: null host buffer");
      if (async) {
        cudaStream_t cs = ic->cstream;
        if (!ic->early_all) {
          CK(cudaEventRecord(ic->ev_pos, s));
          CK(cudaStreamWaitEvent(cs, ic->ev_pos, 0));
          if (!ic->pos_early) CK(cudaMemcpyAsync(out->pos, ic->dpos, ic->pos_bytes, cudaMemcpyDeviceToHost, cs));
          CK(cudaMemcpyAsync(out->vel, ic->dvel, ic->vel_bytes, cudaMemcpyDeviceToHost, cs));
          if (!fields && !ic->ids_early) {
            CK(cudaMemcpyAsync(out->ids, ic->dids, ic->id_bytes, cudaMemcpyDeviceToHost, cs));
            CK(cudaEventRecord(ic->ev_ids, cs));
          }
          CK(cudaEventRecord(ic->ev_copy, cs));
        }
        CK(cudaEventRecord(ic->ev[8], cs));  // the end of the run's last copy
        return MF_OK;
      }
      if (!ic->early_all) {
        if (!ic->pos_early) CK(cudaMemcpyAsync(out->pos, ic->dpos, ic->pos_bytes, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(out->vel, ic->dvel, ic->vel_bytes, cudaMemcpyDeviceToHost, s));
        if (!fields && !ic->ids_early) CK(cudaMemcpyAsync(out->ids, ic->dids, ic->id_bytes, cudaMemcpyDeviceToHost, s));
      }
      if (ic->pos_early) CK(cudaStreamWaitEvent(s, ic->ev_copy, 0));  // the run ends after the streamed copies
    } else {
      out->pos = ic->dpos;
      out->vel = ic->dvel;
      out->ids = ic->dids;
      out->mass = nullptr;  // single-species pipelines carry no per-particle masses
    }
  }
  CK(cudaEventRecord(ic->ev[8], s));
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
    if (uses_shared_sources(p)) {
      const size_t nreal = (p->lpt_order > 2) ? 22 : 7;
      conv = 3 * M * M * (n / 2 + 1) * 2 * ps + nreal * M * M * M * ps;
    } else {
      const int nbuf = (p->convolver == MF_CONV_ORSZAG) ? 2 : 3;
      conv = (size_t)nbuf * M * M * (n / 2 + 1) * 2 * ps + (p->convolver == MF_CONV_ORSZAG ? grid : 0);
    }
  }
  int64_t np; size_t pb, vb, ib;
  output_sizes(p, &np, &pb, &vb, &ib);
  const size_t nk2 = 3 * (size_t)(n / 2) * (n / 2) + 1;
  const size_t pltg = p->plt ? 4 * (size_t)n * n * (n / 2 + 1) * ps : 0;
  size_t two = 0;  // second species, masses, baryon-CDM tables and fields
  if (p->baryons) {
    const bool fl = p->out_kind == MF_OUT_FIELDS;
    const size_t mb = (size_t)np * ((p->pos64 || fl) ? 8 : 4);
    two = pb + vb + ib + (fl ? 1 : 2) * mb + (size_t)(1 << p->lattice) * 3 * n * sizeof(double);
    if (fl) two += 2 * grid_reals(n) * sizeof(double) + 3 * (size_t)n * n * n * 16 + 16;
    if (p->tk_dbc_table || p->tk_tbc_table)
      two += 5 * nk2 * sizeof(double) + grid + ((p->baryon_vrel && p->tk_tbc_table) ? grid : 0) +
             ((fl && p->baryon_vrel) ? grid : 0);
  }
  *bytes = ngrids * grid + conv + pb + vb + ib + 2 * nk2 * sizeof(double) + pltg + two;
  return MF_OK;
}

extern "C" int mf_ic_destroy(mf_ic* ic) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (ic->cstream) cudaStreamSynchronize(ic->cstream);  // copies of an asynchronous run
  if (ic->hstream) cudaStreamSynchronize(ic->hstream);  // a host noise upload
  if (ic->wn) mf_grid_destroy(ic->wn);
  for (auto& g : ic->f)
    if (g) mf_grid_destroy(g);
  for (auto& g : ic->tmp)
    if (g) mf_grid_destroy(g);
  cudaFree(ic->phase);
  cudaFree(ic->qtab);
  cudaFree(ic->plt);
  cudaFree(ic->pltg);
  cudaFree(ic->stage);
  if (ic->conv) mf_conv_destroy(ic->conv);
  cudaFree(ic->rf);
  cudaFree(ic->w3);
  cudaFree(ic->amp);
  cudaFree(ic->dpos);
  cudaFree(ic->dvel);
  cudaFree(ic->dids);
  cudaFree(ic->bpos);
  cudaFree(ic->bvel);
  cudaFree(ic->bids);
  cudaFree(ic->dmass[0]);
  cudaFree(ic->dmass[1]);
  cudaFree(ic->bqtab);
  cudaFree(ic->ampbc);
  if (ic->rho_bc) mf_grid_destroy(ic->rho_bc);
  if (ic->psi_bc) mf_grid_destroy(ic->psi_bc);
  if (ic->rho_e) mf_grid_destroy(ic->rho_e);
  cudaFree(ic->ppt);
  for (auto& e : ic->ev)
    if (e) cudaEventDestroy(e);
  cudaFree(ic->dyn_d);
  cudaFreeHost(ic->dyn_h);
  if (ic->cstream) cudaStreamDestroy(ic->cstream);
  if (ic->hstream) cudaStreamDestroy(ic->hstream);
  for (cudaEvent_t ev : {ic->ev_pos, ic->ev_copy, ic->ev_ids, ic->ev_stage_free, ic->ev_stage_full})
    if (ev) cudaEventDestroy(ev);
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
  for (auto& g : ic->tmp)
    if ((rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &g))) return fail(rc);
  {
    // sub-lattice phase table, generated on the host in extended precision
    const long double pi = 3.141592653589793238462643383279502884L;
    const size_t ps = (p->precision == MF_PREC_F32) ? sizeof(float2) : sizeof(double2);
    std::vector<double> re(4 * n), im(4 * n);
    for (int m = 0; m < 4 * n; ++m) {  // exp(2 pi i m / 4n)
      const long double a = pi * (long double)m / (2.0L * (long double)n);
      re[m] = (double)cosl(a);
      im[m] = (double)sinl(a);
      if (m % n == 0) {  // exact on the axes
        const int q = m / n;
        const double cq[4] = {1, 0, -1, 0}, sq[4] = {0, 1, 0, -1};
        re[m] = cq[q];
        im[m] = sq[q];
      }
    }
    std::vector<unsigned char> h(ps * 4 * n);
    for (int m = 0; m < 4 * n; ++m) {
      if (p->precision == MF_PREC_F32) reinterpret_cast<float2*>(h.data())[m] = make_float2((float)re[m], (float)im[m]);
      else reinterpret_cast<double2*>(h.data())[m] = make_double2(re[m], im[m]);
    }
    cudaError_t e2 = cudaMalloc(&ic->phase, h.size());
    if (e2 == cudaSuccess) e2 = cudaMemcpy(ic->phase, h.data(), h.size(), cudaMemcpyHostToDevice);
    if (e2 != cudaSuccess) return fail(cuda_err(c, e2, "mf_ic_create: phase table"));
    // lattice coordinates (get_unit_r_shifted, grid_fft.hh:242-252) times lunit
    const int ov = 1 << p->lattice;
    std::vector<double> q((size_t)ov * 3 * n);
    for (int ish = 0; ish < ov; ++ish)
      for (int d = 0; d < 3; ++d)
        for (int i = 0; i < n; ++i)
          q[((size_t)ish * 3 + d) * n + i] = ((double)i + kShifts[p->lattice][ish][d]) / (double)n * p->lunit;
    if ((e2 = upload_lattice_table(q, &ic->qtab)) != cudaSuccess)
      return fail(cuda_err(c, e2, "mf_ic_create: lattice table"));
  }
  if (p->plt) {
    PLTTables t;
    ic->plt_ng = p->plt_ngrid ? p->plt_ngrid : 64;
    if ((rc = plt_build_tables(c, p->lattice, ic->plt_ng, &t))) return fail(rc);
    const size_t nkt = t.Dr.size();
    const size_t es = (p->precision == MF_PREC_F32) ? sizeof(float) : sizeof(double);
    std::vector<unsigned char> h(4 * nkt * es);
    const std::vector<double>* src[4] = {&t.Dr, &t.Dth, &t.Dph, &t.Dvf};
    for (int a = 0; a < 4; ++a)
      for (size_t q = 0; q < nkt; ++q) {
        if (es == sizeof(float)) reinterpret_cast<float*>(h.data())[a * nkt + q] = (float)(*src[a])[q];
        else reinterpret_cast<double*>(h.data())[a * nkt + q] = (*src[a])[q];
      }
    cudaError_t e3 = cudaMalloc(&ic->plt, h.size());
    if (e3 == cudaSuccess) e3 = cudaMemcpy(ic->plt, h.data(), h.size(), cudaMemcpyHostToDevice);
    if (e3 != cudaSuccess) return fail(cuda_err(c, e3, "mf_ic_create: PLT tables"));
    const size_t nmode = (size_t)n * n * (n / 2 + 1);
    if ((e3 = cudaMalloc(&ic->pltg, 4 * nmode * es)) != cudaSuccess) return fail(cuda_err(c, e3, "mf_ic_create: PLT gradient"));
    auto launch = [&](auto tag) {
      using T = decltype(tag);
      PLTDev<T> P;
      const T* base = (const T*)ic->plt;
      P.Dr = base;
      P.Dth = base + nkt;
      P.Dph = base + 2 * nkt;
      P.Dvf = base + 3 * nkt;
      P.ng = ic->plt_ng;
      P.mapratio = T((double)ic->plt_ng / (double)n);
      P.inv_mr_L = T(1.0 / ((double)ic->plt_ng / (double)n) / p->boxlen);
      k_plt_grad_table<T><<<blocks_for(nmode), kThreads, 0, c->stream>>>((T*)ic->pltg, n, P);
    };
    if (es == sizeof(float)) launch(float{});
    else launch(double{});
    if ((e3 = cudaGetLastError()) == cudaSuccess) e3 = cudaStreamSynchronize(c->stream);
    if (e3 != cudaSuccess) return fail(cuda_err(c, e3, "mf_ic_create: PLT gradient"));
  }
  if (uses_shared_sources(p)) {
    ic->shared = true;
    const size_t M = 3 * (size_t)n / 2, cs = (p->precision == MF_PREC_F32) ? sizeof(float2) : sizeof(double2);
    const size_t nreal = (p->lpt_order > 2) ? 22 : 7;  // operands + the product-sum scratch fields
    cudaError_t e4 = cudaMalloc(&ic->rf, nreal * M * M * (M / 2) * cs);
    if (e4 == cudaSuccess) e4 = cudaMalloc(&ic->w3, 3 * M * M * (n / 2 + 1) * cs);
    if (e4 != cudaSuccess) return fail(cuda_err(c, e4, "mf_ic_create: shared-source buffers"));
  } else if (p->lpt_order > 1) {
    if ((rc = mf_conv_create(c, n, p->boxlen, p->precision, p->convolver, &ic->conv))) return fail(rc);
  }
  ic->nk2 = 3 * (n / 2) * (n / 2) + 1;
  cudaError_t e = cudaMalloc(&ic->amp, sizeof(double) * 2 * ic->nk2);
  if (e != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: amplitude table"));
  if (p->tk_table) {  // tabulated T(k) of any transfer plugin, one value per integer k^2
    e = cudaMemcpy(ic->amp + ic->nk2, p->tk_table, sizeof(double) * ic->nk2, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: T(k) table"));
    ic->has_tk = true;
  }
  if ((e = cudaHostAlloc((void**)&ic->dyn_h, sizeof(ICDyn), cudaHostAllocDefault)) != cudaSuccess)
    return fail(cuda_err(c, e, "mf_ic_create: parameter block"));
  std::memset(ic->dyn_h, 0, sizeof(ICDyn));
  if ((e = cudaMalloc((void**)&ic->dyn_d, sizeof(ICDyn))) != cudaSuccess)
    return fail(cuda_err(c, e, "mf_ic_create: parameter block"));
  fill_dyn(ic);
  // twiddle tables of every length the pipeline uses, built now so that a
  // run can be recorded into a graph
  {
    const int M = (p->convolver == MF_CONV_ORSZAG) ? 3 * n / 2 : n;
    const int lens[4] = {n, n / 2, M, M / 2};
    for (int L : lens) {
      const void* t = (p->precision == MF_PREC_F32) ? (const void*)c->tw.get<float>(L, c->stream)
                                                     : (const void*)c->tw.get<double>(L, c->stream);
      if (!t) return fail(set_err(c, MF_ERR_OOM, "mf_ic_create: twiddle tables"));
    }
  }
  output_sizes(p, &ic->npart, &ic->pos_bytes, &ic->vel_bytes, &ic->id_bytes);
  if ((e = cudaMalloc(&ic->dpos, ic->pos_bytes)) != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: positions"));
  if ((e = cudaMalloc(&ic->dvel, ic->vel_bytes)) != cudaSuccess) return fail(cuda_err(c, e, "mf_ic_create: velocities"));
  if (ic->id_bytes && (e = cudaMalloc(&ic->dids, ic->id_bytes)) != cudaSuccess)
    return fail(cuda_err(c, e, "mf_ic_create: ids"));
  if (p->baryons) {
    ic->p.tk_dbc_table = ic->p.tk_tbc_table = nullptr;  // host tables are copied, not kept
    const bool fields = p->out_kind == MF_OUT_FIELDS;
    // particles: per-particle masses of both species; fields: the dark
    // matter's mass field (n^3 doubles) and the baryons' Eulerian density
    // (first n^3 doubles of the position buffer) and velocities
    ic->mass_bytes = fields ? (size_t)ic->npart * 8 : (size_t)ic->npart * (p->pos64 ? 8 : 4);
    if ((e = cudaMalloc(&ic->bpos, ic->pos_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&ic->bvel, ic->vel_bytes)) != cudaSuccess ||
        (ic->id_bytes && (e = cudaMalloc(&ic->bids, ic->id_bytes)) != cudaSuccess) ||
        (e = cudaMalloc(&ic->dmass[0], ic->mass_bytes)) != cudaSuccess ||
        (!fields && (e = cudaMalloc(&ic->dmass[1], ic->mass_bytes)) != cudaSuccess))
      return fail(cuda_err(c, e, "mf_ic_create: baryon particles"));
    if (fields) {
      const size_t n3 = (size_t)n * n * n;
      if ((e = cudaMalloc(&ic->ppt, 2 * grid_reals(n) * sizeof(double) + 3 * n3 * sizeof(double2) + 16)) != cudaSuccess)
        return fail(cuda_err(c, e, "mf_ic_create: Eulerian-branch buffers"));
    }
    // secondary-lattice coordinates: get_unit_r_shifted with lattice_shifts[ish]
    // + second_lattice_shift (particle_generator.hh:531)
    const int ov = 1 << p->lattice;
    std::vector<double> q((size_t)ov * 3 * n);
    for (int ish = 0; ish < ov; ++ish)
      for (int d = 0; d < 3; ++d)
        for (int i = 0; i < n; ++i)
          q[((size_t)ish * 3 + d) * n + i] =
              ((double)i + (kShifts[p->lattice][ish][d] + kSecondShift[p->lattice][d])) / (double)n * p->lunit;
    if ((e = upload_lattice_table(q, &ic->bqtab)) != cudaSuccess)
      return fail(cuda_err(c, e, "mf_ic_create: secondary lattice table"));
    const bool has_d = p->tk_dbc_table != nullptr;
    const bool has_t = p->tk_tbc_table != nullptr;
    if (has_d || has_t) {
      const size_t nk2 = (size_t)ic->nk2;
      // [amp_dbc, amp_tbc, amp_dbc without vbc, T_delta_bc, T_theta_bc]
      if ((e = cudaMalloc(&ic->ampbc, sizeof(double) * 5 * nk2)) != cudaSuccess)
        return fail(cuda_err(c, e, "mf_ic_create: baryon-CDM tables"));
      if (has_d) {
        if ((e = cudaMemcpy(ic->ampbc + 3 * nk2, p->tk_dbc_table, sizeof(double) * nk2, cudaMemcpyHostToDevice)) !=
            cudaSuccess)
          return fail(cuda_err(c, e, "mf_ic_create: T_delta_bc table"));
        ic->tdbc_d = ic->ampbc + 3 * nk2;
      }
      if (has_t) {
        if ((e = cudaMemcpy(ic->ampbc + 4 * nk2, p->tk_tbc_table, sizeof(double) * nk2, cudaMemcpyHostToDevice)) !=
            cudaSuccess)
          return fail(cuda_err(c, e, "mf_ic_create: T_theta_bc table"));
        ic->ttbc_d = ic->ampbc + 4 * nk2;
      }
      // rho_bc feeds the masses; psi_bc only with the relative-velocity mode
      if ((rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &ic->rho_bc))) return fail(rc);
      if (p->baryon_vrel && has_t && (rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &ic->psi_bc)))
        return fail(rc);
      // the Eulerian branch of field output reads delta_bc without the relative-velocity amplitude
      if (fields && p->baryon_vrel && (rc = mf_grid_create(c, n, p->boxlen, p->precision, MF_SPACE_K, &ic->rho_e)))
        return fail(rc);
    }
  }
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
  if (location == MF_LOC_HOST && ic->p.precision == MF_PREC_F64) {
    // rows of n doubles into the padded rows of n+2: one pitched copy
    e = cudaMemcpy2DAsync(ic->wn->d, (size_t)(n + 2) * sizeof(double), noise, (size_t)n * sizeof(double),
                          (size_t)n * sizeof(double), (size_t)n * n, cudaMemcpyHostToDevice, c->stream);
  } else if (location == MF_LOC_HOST) {
    // FP32 grid: through a staging buffer kept by the pipeline (allocated at
    // the first host upload).  The copy runs on the upload stream as soon as
    // the previous upload has been converted, i.e. while the runs queued
    // before it compute; the conversion into the grid is stream-ordered
    if (!ic->stage && (e = cudaMalloc((void**)&ic->stage, n3 * sizeof(double))) != cudaSuccess)
      return cuda_err(c, e, "mf_ic_set_noise: staging buffer");
    if (!ic->hstream) {
      e = cudaStreamCreateWithFlags(&ic->hstream, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ic->ev_stage_free, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ic->ev_stage_full, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_err(c, e, "mf_ic_set_noise: upload stream");
      e = cudaEventRecord(ic->ev_stage_free, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ic->hstream, ic->ev_stage_free, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ic->stage, noise, n3 * sizeof(double), cudaMemcpyHostToDevice, ic->hstream);
    if (e == cudaSuccess) e = cudaEventRecord(ic->ev_stage_full, ic->hstream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, ic->ev_stage_full, 0);
    if (e == cudaSuccess) e = pw_fill_from_f64<float>((float*)ic->wn->d, ic->stage, n, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ic->ev_stage_free, c->stream);
  } else {
    e = (ic->p.precision == MF_PREC_F64) ? pw_fill_from_f64<double>((double*)ic->wn->d, noise, n, c->stream)
                                         : pw_fill_from_f64<float>((float*)ic->wn->d, noise, n, c->stream);
  }
  if (e != cudaSuccess) return cuda_err(c, e, "mf_ic_set_noise");
  ic->wn->space = MF_SPACE_R;
  ic->noise_set = true;
  ic->noise_seeded = false;
  return MF_OK;
}

extern "C" int mf_ic_set_noise_seed(mf_ic* ic, uint64_t seed) {
  if (!ic) return MF_ERR_ARG;
  ic->dyn_h->seed = (unsigned long long)seed;
  ic->noise_seeded = true;
  ic->noise_set = false;
  return MF_OK;
}

extern "C" int mf_ic_set_cosmology(mf_ic* ic, const mf_cosmo_scalars* cosmo) {
  if (!ic || !cosmo) return MF_ERR_ARG;
  if (!(cosmo->pnorm > 0) || !(cosmo->Dplus > 0)) return set_err(ic->ctx, MF_ERR_ARG, "mf_ic_set_cosmology: bad scalars");
  if (ic->has_tk || ic->ampbc)
    return set_err(ic->ctx, MF_ERR_STATE, "mf_ic_set_cosmology: the pipeline uses a tabulated T(k)");
  ic->p.cosmo = *cosmo;
  fill_dyn(ic);
  return MF_OK;
}

extern "C" int mf_ic_enqueue(mf_ic* ic) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  cudaSetDevice(c->device);
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(c->stream, &st);
  if (e != cudaSuccess) return cuda_err(c, e, "mf_ic_enqueue: capture status");
  const bool cap = (st == cudaStreamCaptureStatusActive);
  if (cap && !ic->noise_seeded)
    return set_err(c, MF_ERR_STATE, "mf_ic_enqueue: a recorded pipeline needs the device noise generator (mf_ic_set_noise_seed)");
  if (!ic->noise_set && !ic->noise_seeded) return set_err(c, MF_ERR_STATE, "mf_ic_enqueue: white noise not set");
  c->capturing = cap;
  const int rc = (ic->p.precision == MF_PREC_F64) ? enqueue_impl<double>(ic) : enqueue_impl<float>(ic);
  c->capturing = false;
  if (!cap) ic->noise_set = false;  // the uploaded grid is consumed (transformed in place)
  return rc;
}

namespace {
void reset_early(mf_ic* ic) {
  ic->early = nullptr;
  ic->early_all = false;
  ic->pos_early = false;
  ic->ids_early = false;
}

// the copy stream and its events, created at the first host hand-off
int make_copy_stream(mf_ic* ic, const char* where) {
  cudaError_t e = cudaSuccess;
  if (!ic->cstream) e = cudaStreamCreateWithFlags(&ic->cstream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !ic->ev_pos) e = cudaEventCreateWithFlags(&ic->ev_pos, cudaEventDisableTiming);
  if (e == cudaSuccess && !ic->ev_copy) e = cudaEventCreateWithFlags(&ic->ev_copy, cudaEventDisableTiming);
  if (e == cudaSuccess && !ic->ev_ids) e = cudaEventCreateWithFlags(&ic->ev_ids, cudaEventDisableTiming);
  return e == cudaSuccess ? MF_OK : cuda_err(ic->ctx, e, where);
}

bool host_buffers(const mf_ic* ic, const mf_particles* out) {
  return out && out->location == MF_LOC_HOST && out->pos && out->vel &&
         (ic->p.out_kind == MF_OUT_FIELDS || out->ids);
}

// a host hand-off runs on a second stream and cannot be recorded into a graph
int refuse_capture(mf_ic* ic, const char* where) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ic->ctx->stream, &st) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ic->ctx, MF_ERR_STATE, where);
  }
  return st == cudaStreamCaptureStatusNone ? MF_OK : set_err(ic->ctx, MF_ERR_STATE, where);
}
}  // namespace

extern "C" int mf_ic_run(mf_ic* ic, mf_particles* out) {
  if (!ic) return MF_ERR_ARG;
  if (ic->p.baryons) return set_err(ic->ctx, MF_ERR_ARG, "mf_ic_run: a two-species pipeline runs with mf_ic_run_species");
  if (!ic->noise_set && !ic->noise_seeded) return set_err(ic->ctx, MF_ERR_STATE, "mf_ic_run: white noise not set");
  reset_early(ic);
  if (host_buffers(ic, out)) {
    int rc = refuse_capture(ic, "mf_ic_run: a run into host buffers cannot be captured (use mf_ic_enqueue)");
    if (rc == MF_OK) rc = make_copy_stream(ic, "mf_ic_run: copy stream");
    if (rc != MF_OK) return rc;
    ic->early = out;
  }
  int rc = mf_ic_enqueue(ic);
  if (rc == MF_OK) rc = handoff(ic, out, false);
  if (rc == MF_OK) rc = check_device_error(ic->ctx);
  else cudaStreamSynchronize(ic->ctx->stream);
  if (ic->cstream) cudaStreamSynchronize(ic->cstream);
  reset_early(ic);
  return rc;
}

extern "C" int mf_ic_run_async(mf_ic* ic, const mf_particles* out) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  if (ic->p.baryons) return set_err(c, MF_ERR_ARG, "mf_ic_run_async: a two-species pipeline runs with mf_ic_run_species");
  if (!host_buffers(ic, out)) return set_err(c, MF_ERR_ARG, "mf_ic_run_async: host buffers expected");
  if (!ic->noise_set && !ic->noise_seeded) return set_err(c, MF_ERR_STATE, "mf_ic_run_async: white noise not set");
  int rc = refuse_capture(ic, "mf_ic_run_async: a run into host buffers cannot be captured (use mf_ic_enqueue)");
  if (rc == MF_OK) rc = make_copy_stream(ic, "mf_ic_run_async: copy stream");
  if (rc != MF_OK) return rc;
  reset_early(ic);
  ic->early_out = *out;
  ic->early = &ic->early_out;
  rc = mf_ic_enqueue(ic);
  if (rc == MF_OK) rc = handoff(ic, &ic->early_out, true);
  reset_early(ic);
  if (rc != MF_OK) {  // nothing of a failed run stays in flight
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(ic->cstream);
  }
  return rc;
}

extern "C" int mf_ic_wait(mf_ic* ic) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  cudaSetDevice(c->device);
  int rc = check_device_error(c);
  if (ic->cstream) {
    const cudaError_t e = cudaStreamSynchronize(ic->cstream);
    if (rc == MF_OK && e != cudaSuccess) rc = cuda_err(c, e, "mf_ic_wait: copy stream");
  }
  return rc;
}

extern "C" int mf_ic_particles(mf_ic* ic, mf_particles* out) {
  if (!ic || !out) return MF_ERR_ARG;
  out->pos = ic->dpos;
  out->vel = ic->dvel;
  out->ids = ic->dids;
  out->npart = ic->npart;
  out->location = MF_LOC_DEVICE;
  out->mass = ic->dmass[0];  // dark-matter masses of a two-species pipeline, else null
  return MF_OK;
}

namespace mf {
const mf_ic_params* ic_params(const mf_ic* ic) { return &ic->p; }
}  // namespace mf

extern "C" int mf_ic_particles_species(mf_ic* ic, int species, mf_particles* out) {
  if (!ic || !out || species < MF_SPECIES_DM || species > (ic->p.baryons ? MF_SPECIES_BARYON : MF_SPECIES_DM))
    return MF_ERR_ARG;
  const bool b = species == MF_SPECIES_BARYON;
  out->pos = b ? ic->bpos : ic->dpos;
  out->vel = b ? ic->bvel : ic->dvel;
  out->ids = b ? ic->bids : ic->dids;
  out->mass = ic->dmass[b ? 1 : 0];
  out->npart = ic->npart;
  out->location = MF_LOC_DEVICE;
  return MF_OK;
}

extern "C" int mf_ic_run_species(mf_ic* ic, mf_particles* out, int nspecies) {
  if (!ic) return MF_ERR_ARG;
  mf_ctx* c = ic->ctx;
  if (!ic->p.baryons) return set_err(c, MF_ERR_ARG, "mf_ic_run_species: the pipeline has one species (use mf_ic_run)");
  if (!out || nspecies != 2) return set_err(c, MF_ERR_ARG, "mf_ic_run_species: two species expected");
  if (!ic->noise_set && !ic->noise_seeded) return set_err(c, MF_ERR_STATE, "mf_ic_run_species: white noise not set");
  const bool fields = ic->p.out_kind == MF_OUT_FIELDS;
  // bytes handed over per species: pos, vel, ids, mass (field output: the
  // dark matter's fields and mass field, the baryons' density and velocities)
  const size_t n3 = (size_t)ic->p.ngrid * ic->p.ngrid * ic->p.ngrid;
  const size_t bytes[2][4] = {{ic->pos_bytes, ic->vel_bytes, fields ? 0 : ic->id_bytes, ic->mass_bytes},
                              {fields ? n3 * sizeof(double) : ic->pos_bytes, ic->vel_bytes, fields ? 0 : ic->id_bytes,
                               fields ? 0 : ic->mass_bytes}};
  for (int sp = 0; sp < 2; ++sp) {
    if (out[sp].location != MF_LOC_HOST) continue;
    void* const h[4] = {out[sp].pos, out[sp].vel, out[sp].ids, out[sp].mass};
    for (int a = 0; a < 4; ++a)
      if (bytes[sp][a] && !h[a]) return set_err(c, MF_ERR_ARG, "mf_ic_run_species: null host buffer");
  }
  ic->early = nullptr;  // the hand-off happens after the run
  ic->early_all = false;
  ic->pos_early = false;
  ic->ids_early = false;
  int rc = mf_ic_enqueue(ic);
  cudaError_t e = cudaSuccess;
  for (int sp = 0; sp < 2 && rc == MF_OK; ++sp) {
    mf_particles dev{};
    mf_ic_particles_species(ic, sp, &dev);
    mf_particles& o = out[sp];
    o.npart = ic->npart;
    if (o.location == MF_LOC_HOST) {
      const void* src[4] = {dev.pos, dev.vel, dev.ids, dev.mass};
      void* dst[4] = {o.pos, o.vel, o.ids, o.mass};
      for (int a = 0; a < 4 && e == cudaSuccess; ++a)
        if (bytes[sp][a]) e = cudaMemcpyAsync(dst[a], src[a], bytes[sp][a], cudaMemcpyDeviceToHost, c->stream);
    } else {
      o = dev;
    }
  }
  if (rc == MF_OK && e == cudaSuccess) e = cudaEventRecord(ic->ev[8], c->stream);
  if (rc == MF_OK && e != cudaSuccess) rc = cuda_err(c, e, "mf_ic_run_species: hand-off");
  if (rc == MF_OK) rc = check_device_error(c);
  else cudaStreamSynchronize(c->stream);
  return rc;
}

extern "C" int mf_ic_mass_bytes(const mf_ic_params* p, size_t* bytes) {
  int rc = check_params(p);
  if (rc) return rc;
  if (!bytes) return MF_ERR_ARG;
  int64_t np; size_t pb, vb, ib;
  output_sizes(p, &np, &pb, &vb, &ib);
  *bytes = !p->baryons ? 0 : (size_t)np * ((p->pos64 || p->out_kind == MF_OUT_FIELDS) ? 8 : 4);
  return MF_OK;
}

extern "C" int mf_ic_context(mf_ic* ic, mf_ctx** out) {
  if (!ic || !out) return MF_ERR_ARG;
  *out = ic->ctx;
  return MF_OK;
}

extern "C" int mf_ic_stage_times(const mf_ic* ic, double* ms) {
  if (!ic || !ms) return MF_ERR_ARG;
  for (int i = 0; i < 8; ++i) {
    float t = 0;
    if (cudaEventElapsedTime(&t, ic->ev[i], ic->ev[i + 1]) != cudaSuccess) {
      t = -1;             // a stage the last run did not record
      cudaGetLastError();  // (not an error of the next call's)
    }
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
