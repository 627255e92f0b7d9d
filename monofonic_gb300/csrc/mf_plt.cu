// PLT tables: host restatement of lattice_gradient::init_D
// (include/particle_plt.hh:68-515) with the mesh transforms on the device.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/monofonic_gb300_ic.h"
#include "mf_plt.h"

namespace mf {
namespace {

using V3 = std::array<double, 3>;
using M3 = std::array<double, 9>;  // row-major

V3 mul(const M3& A, const V3& v) {
  return V3{A[0] * v[0] + A[1] * v[1] + A[2] * v[2], A[3] * v[0] + A[4] * v[1] + A[5] * v[2],
            A[6] * v[0] + A[7] * v[1] + A[8] * v[2]};
}
double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix; eigenvalues
// ascending (as gsl_eigen_symmv + GSL_EIGEN_SORT_VAL_ASC, mat3.hh:169-190),
// eigenvectors as columns of V
void eigen3(M3 A, V3& ev, M3& V) {
  V = M3{1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    if (off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const double apq = A[3 * p + q];
        if (apq == 0.0) continue;
        const double app = A[3 * p + p], aqq = A[3 * q + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {  // A <- J^T A J
          const double akp = A[3 * k + p], akq = A[3 * k + q];
          A[3 * k + p] = c * akp - s * akq;
          A[3 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = A[3 * p + k], aqk = A[3 * q + k];
          A[3 * p + k] = c * apk - s * aqk;
          A[3 * q + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[3 * k + p], vkq = V[3 * k + q];
          V[3 * k + p] = c * vkp - s * vkq;
          V[3 * k + q] = s * vkp + c * vkq;
        }
      }
  }
  ev = V3{A[0], A[4], A[8]};
  // sort ascending with the eigenvector columns
  int idx[3] = {0, 1, 2};
  std::sort(idx, idx + 3, [&](int a, int b) { return ev[a] < ev[b]; });
  const V3 e0 = ev;
  const M3 V0 = V;
  for (int c2 = 0; c2 < 3; ++c2) {
    ev[c2] = e0[idx[c2]];
    for (int r = 0; r < 3; ++r) V[3 * r + c2] = V0[3 * r + idx[c2]];
  }
}

struct Lattice {
  M3 B, R;
  int IR[9];
  std::vector<V3> normals;
  int charge_fac;
};

// Bravais, reciprocal and inverse-reciprocal matrices and FBZ normals
// (particle_plt.hh:76-164); RSC uses the SC set as in the reference
Lattice lattice_set(int lattice) {
  const double pi = M_PI, twopi = 2 * M_PI, fourpi = 4 * M_PI;
  Lattice L;
  if (lattice == 1) {
    L.charge_fac = 2;
    L.B = M3{1, 0, 0.5, 0, 1, 0.5, 0, 0, 0.5};
    L.R = M3{twopi, 0, 0, 0, twopi, 0, -twopi, -twopi, fourpi};
    const int ir[9] = {2, 0, 0, 0, 2, 0, 1, 1, 1};
    std::copy(ir, ir + 9, L.IR);
    L.normals = {{0, pi, pi},  {0, -pi, pi},  {0, pi, -pi},  {0, -pi, -pi}, {pi, 0, pi},  {-pi, 0, pi},
                 {pi, 0, -pi}, {-pi, 0, -pi}, {pi, pi, 0},   {-pi, pi, 0},  {pi, -pi, 0}, {-pi, -pi, 0}};
  } else if (lattice == 2) {
    L.charge_fac = 4;
    L.B = M3{0, 0.5, 0, 0.5, 0, 1, 0.5, 0.5, 0};
    L.R = M3{-fourpi, fourpi, twopi, 0, 0, twopi, fourpi, 0, -twopi};
    const int ir[9] = {0, 1, 1, 1, 0, 1, 0, 2, 0};
    std::copy(ir, ir + 9, L.IR);
    L.normals = {{twopi, 0, 0}, {-twopi, 0, 0}, {0, twopi, 0}, {0, -twopi, 0}, {0, 0, twopi},
                 {0, 0, -twopi}, {pi, pi, pi},  {pi, pi, -pi},  {pi, -pi, pi},  {pi, -pi, -pi},
                 {-pi, pi, pi},  {-pi, pi, -pi}, {-pi, -pi, pi}, {-pi, -pi, -pi}};
  } else {
    L.charge_fac = 1;
    L.B = M3{1, 0, 0, 0, 1, 0, 0, 0, 1};
    L.R = M3{twopi, 0, 0, 0, twopi, 0, 0, 0, twopi};
    const int ir[9] = {2, 0, 0, 0, 2, 0, 0, 0, 2};
    std::copy(ir, ir + 9, L.IR);
    L.normals = {{pi, 0, 0}, {-pi, 0, 0}, {0, pi, 0}, {0, -pi, 0}, {0, 0, pi}, {0, 0, -pi}};
  }
  return L;
}

}  // namespace

int plt_build_tables(mf_ctx* c, int lattice, int ng, PLTTables* out) {
  if (!grid_size_supported(ng)) return set_err(c, MF_ERR_SHAPE, "PLT mesh size not supported");
  const Lattice LT = lattice_set(lattice);
  const double pi = M_PI, fourpi = 4 * M_PI, twopi = 2 * M_PI;
  const double sqrtpi = std::sqrt(M_PI), pi32 = std::pow(M_PI, 1.5);
  const int nl = ng;
  const double dx = 1.0 / nl;
  const double eta = 4.0, alpha = 1.0 / std::sqrt(2.0) / eta, alpha2 = alpha * alpha, alpha3 = alpha2 * alpha;
  const double charge = 1.0 / std::pow(double(nl), 3) / LT.charge_fac;
  const double fft_norm = 1.0 / std::pow(double(nl), 3.0);
  const double fft_norm12 = 1.0 / std::pow(double(nl), 1.5);
  const size_t n3 = (size_t)nl * nl * nl;

  // ---- Ewald sums of the dynamical matrix in real space (particle_plt.hh:167-260)
  std::vector<double> D6[6];
  for (auto& d : D6) d.assign(n3, 0.0);
  auto work = [&](int i0, int i1) {
    for (int i = i0; i < i1; ++i)
      for (int j = 0; j < nl; ++j)
        for (int k = 0; k < nl; ++k) {
          V3 ar = mul(LT.B, V3{dx * i, dx * j, dx * k});
          for (auto& a : ar) a = std::fmod(2.0 + a, 1.0);  // wrap_abs (vec3.hh:111-114)
          double M[9] = {0};
          for (int ix = -3; ix <= 3; ++ix)
            for (int iy = -3; iy <= 3; ++iy)
              for (int iz = -3; iz <= 3; ++iz) {
                const V3 bn = mul(LT.B, V3{double(ix), double(iy), double(iz)});
                const V3 d{ar[0] - bn[0], ar[1] - bn[1], ar[2] - bn[2]};
                const double r = std::sqrt(dot(d, d));
                if (r < 1e-14) continue;
                const double r2 = r * r, r3 = r2 * r, r5 = r3 * r2;
                const double K1 = -alpha3 / pi32 * std::exp(-alpha2 * r2) / r2;
                const double K2 = (std::erfc(alpha * r) + 2.0 * alpha / sqrtpi * std::exp(-alpha2 * r2) * r) / fourpi;
                for (int mu = 0; mu < 3; ++mu)
                  for (int nu = mu; nu < 3; ++nu) {
                    const double dd = d[mu] * d[nu] * K1 + ((mu == nu ? 1.0 : 0.0) / r3 - 3.0 * (d[mu] * d[nu]) / r5) * K2;
                    M[3 * mu + nu] += dd;
                    if (mu != nu) M[3 * nu + mu] += dd;
                  }
              }
          for (int ix = -3; ix <= 3; ++ix)
            for (int iy = -3; iy <= 3; ++iy)
              for (int iz = -3; iz <= 3; ++iz) {
                if (std::abs(ix) + std::abs(iy) + std::abs(iz) == 0) continue;
                const V3 ak = mul(LT.R, V3{double(ix) / nl, double(iy) / nl, double(iz) / nl});
                const double kmod2 = dot(ak, ak);
                const double term = std::exp(-kmod2 / (4 * alpha2)) * std::cos(dot(ak, ar)) / kmod2 * fft_norm;
                for (int mu = 0; mu < 3; ++mu)
                  for (int nu = mu; nu < 3; ++nu) {
                    const double dd = ak[mu] * ak[nu] * term;
                    M[3 * mu + nu] += dd;
                    if (mu != nu) M[3 * nu + mu] += dd;
                  }
              }
          const size_t cidx = ((size_t)i * nl + j) * nl + k;
          D6[0][cidx] = M[0] * charge;
          D6[1][cidx] = M[1] * charge;
          D6[2][cidx] = M[2] * charge;
          D6[3][cidx] = M[4] * charge;
          D6[4][cidx] = M[5] * charge;
          D6[5][cidx] = M[8] * charge;
        }
  };
  {
    const int nt = std::max(1, std::min<int>(nl, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t * nl / nt, (t + 1) * nl / nt);
    for (auto& t : th) t.join();
  }
  // r = 0 with the background density (particle_plt.hh:263-269)
  D6[0][0] = 1.0 / 3.0; D6[1][0] = 0.0; D6[2][0] = 0.0;
  D6[3][0] = 1.0 / 3.0; D6[4][0] = 0.0; D6[5][0] = 1.0 / 3.0;

  // ---- forward transforms on the device (unitary), real parts kept
  const int nk = nl / 2 + 1;
  const size_t nkt = (size_t)nl * nl * nk;
  std::vector<double> Dk[6];
  {
    mf_grid* g = nullptr;
    int rc = mf_grid_create(c, nl, 1.0, MF_PREC_F64, MF_SPACE_R, &g);
    if (rc) return rc;
    std::vector<double> pad(grid_reals(nl));
    for (int a = 0; a < 6; ++a) {
      rc = mf_grid_fill_real64(g, D6[a].data());
      if (!rc) rc = mf_grid_fft_forward(g, 1);
      if (!rc) rc = mf_grid_download(g, pad.data());
      g->space = MF_SPACE_R;
      if (rc) { mf_grid_destroy(g); return rc; }
      Dk[a].resize(nkt);
      for (size_t q = 0; q < nkt; ++q) Dk[a][q] = pad[2 * q];
    }
    mf_grid_destroy(g);
  }

  // ---- eigen-decomposition and first-Brillouin-zone mapping (:295-390)
  auto kcomp64 = [&](int idx) { return (double(idx) - double(idx > nl / 2) * nl) * twopi; };
  std::vector<double> T1r(nkt), T1i(nkt), T2r(nkt), T2i(nkt), T3r(nkt), T3i(nkt);
  for (size_t q = 0; q < nkt; ++q) {
    T1r[q] = Dk[0][q]; T1i[q] = Dk[1][q];
    T2r[q] = Dk[2][q]; T2i[q] = Dk[3][q];
    T3r[q] = Dk[4][q]; T3i[q] = Dk[5][q];
  }
  std::map<std::tuple<int, int, int>, size_t> iimap;
  auto check_FBZ = [&](const V3& v) {
    for (const auto& nrm : LT.normals)
      if (dot(nrm, v) > 1.0001 * dot(nrm, nrm)) return false;
    return true;
  };
  for (int i = 0; i < nl; ++i)
    for (int j = 0; j < nl; ++j)
      for (int k = 0; k < nk; ++k) {
        const size_t q = ((size_t)i * nl + j) * nk + k;
        const V3 kv{kcomp64(i), kcomp64(j), kcomp64(k)};
        M3 D{Dk[0][q] / fft_norm12, Dk[1][q] / fft_norm12, Dk[2][q] / fft_norm12,
             Dk[1][q] / fft_norm12, Dk[3][q] / fft_norm12, Dk[4][q] / fft_norm12,
             Dk[2][q] / fft_norm12, Dk[4][q] / fft_norm12, Dk[5][q] / fft_norm12};
        V3 ev;
        M3 Vm;
        eigen3(D, ev, Vm);
        V3 e3{Vm[2], Vm[5], Vm[8]};
        for (auto& x : e3) x /= (twopi * ng);
        const V3 ar{kv[0] / (twopi * ng), kv[1] / (twopi * ng), kv[2] / (twopi * ng)};
        const V3 a = mul(LT.R, ar);
        for (int l1 = -1; l1 <= 1; ++l1)
          for (int l2 = -1; l2 <= 1; ++l2)
            for (int l3 = -1; l3 <= 1; ++l3)
              for (int is = 0; is <= 1; ++is) {
                const double sg = 2.0 * is - 1.0;
                const V3 rs = mul(LT.R, V3{double(l1), double(l2), double(l3)});
                const V3 vk{sg * a[0] + rs[0], sg * a[1] + rs[1], sg * a[2] + rs[2]};
                if (check_FBZ(vk)) {
                  const int ix = (int)std::round(vk[0] * ng / twopi);
                  const int iy = (int)std::round(vk[1] * ng / twopi);
                  const int iz = (int)std::round(vk[2] * ng / twopi);
                  iimap.insert({std::make_tuple(ix, iy, iz), q});
                  T1r[q] = ev[2]; T1i[q] = ev[1];
                  T2r[q] = ev[0]; T2i[q] = e3[0];
                  T3r[q] = e3[1]; T3i[q] = e3[2];
                }
              }
      }

  // ---- neighbour averaging onto the regular mesh (:401-458)
  std::vector<double> Dxx(nkt, 0.0), Dxy(nkt, 0.0), Dyy(nkt, 0.0), Dyz(nkt, 0.0), Dzz(nkt, 0.0);
  auto is_in = [&](int i, int j, int k) {
    for (int r = 0; r < 3; ++r)
      if ((LT.IR[3 * r] * i + LT.IR[3 * r + 1] * j + LT.IR[3 * r + 2] * k) % 2 != 0) return false;
    return true;
  };
  for (int i = 0; i < nl; ++i)
    for (int j = 0; j < nl; ++j)
      for (int k = 0; k < nk; ++k) {
        const size_t q0 = ((size_t)i * nl + j) * nk + k;
        const int ii = (i > nl / 2) ? i - nl : i, jj = (j > nl / 2) ? j - nl : j, kk = (k > nl / 2) ? k - nl : k;
        const V3 kvv{double(ii), double(jj), double(kk)};
        auto align = [&](V3 v) {
          if (dot(v, kvv) < 0.0) for (auto& x : v) x = -x;
          return v;
        };
        V3 l{0, 0, 0}, v{0, 0, 0};
        if (!is_in(i, j, k)) {
          int count = 0;
          const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
          for (const auto& o : nb) {
            auto it = iimap.find(std::make_tuple(ii + o[0], jj + o[1], kk + o[2]));
            if (it == iimap.end()) continue;
            const size_t q = it->second;
            ++count;
            l[0] += T1r[q]; l[1] += T1i[q]; l[2] += T2r[q];
            const V3 a = align(V3{T2i[q], T3r[q], T3i[q]});
            v[0] += a[0]; v[1] += a[1]; v[2] += a[2];
          }
          for (auto& x : l) x /= double(count);
          for (auto& x : v) x /= double(count);
        } else {
          auto it = iimap.find(std::make_tuple(ii, jj, kk));
          if (it != iimap.end()) {
            const size_t q = it->second;
            l = V3{T1r[q], T1i[q], T2r[q]};
            v = align(V3{T2i[q], T3r[q], T3i[q]});
          }
        }
        Dxx[q0] = l[0];
        Dxy[q0] = l[1];
        Dyy[q0] = v[0];
        Dyz[q0] = v[1];
        Dzz[q0] = v[2];
      }

  // ---- projection onto spherical unit vectors (:461-487)
  out->ng = ng;
  out->lattice = lattice;
  out->Dr.assign(nkt, 1.0);
  out->Dth.assign(nkt, 0.0);
  out->Dph.assign(nkt, 0.0);
  out->Dvf.assign(nkt, 1.0);
  for (int i = 0; i < nl; ++i)
    for (int j = 0; j < nl; ++j)
      for (int k = 0; k < nk; ++k) {
        const size_t q = ((size_t)i * nl + j) * nk + k;
        const V3 kv{kcomp64(i), kcomp64(j), kcomp64(k)};
        const double mu1 = Dxx[q];
        V3 e1{Dyy[q], Dyz[q], Dzz[q]};
        const double en = std::sqrt(dot(e1, e1));
        for (auto& x : e1) x /= en;
        const double kr = std::sqrt(dot(kv, kv));
        const double kphi = kr > 0.0 ? std::atan2(kv[1], kv[0]) : 0.0;
        const double kth = kr > 0.0 ? std::acos(kv[2] / kr) : 0.0;
        const double st = std::sin(kth), ct = std::cos(kth), sp = std::sin(kphi), cp = std::cos(kphi);
        const V3 e_r{st * cp, st * sp, ct}, e_t{ct * cp, ct * sp, -st}, e_p{-sp, cp, 0.0};
        double renorm = dot(e1, e_r);
        if (renorm < 0.01) renorm = 1.0;
        out->Dr[q] = 1.0;
        out->Dth[q] = dot(e1, e_t) / renorm;
        out->Dph[q] = dot(e1, e_p) / renorm;
        out->Dvf[q] = 1.0 / (0.25 * (std::sqrt(1. + 24 * mu1) - 1.));
      }
  out->Dvf[0] = 1.0;
  out->Dr[0] = 1.0;
  out->Dth[0] = 0.0;
  out->Dph[0] = 0.0;
  (void)pi;
  return MF_OK;
}

}  // namespace mf

extern "C" int mf_plt_tables(mf_ctx* c, int lattice, int ng, double* Dr, double* Dth, double* Dph, double* Dvf) {
  if (!c || !Dr || !Dth || !Dph || !Dvf) return MF_ERR_ARG;
  if (lattice < MF_LATTICE_SC || lattice > MF_LATTICE_RSC) return MF_ERR_ARG;
  cudaSetDevice(c->device);
  mf::PLTTables t;
  int rc = mf::plt_build_tables(c, lattice, ng, &t);
  if (rc) return rc;
  std::copy(t.Dr.begin(), t.Dr.end(), Dr);
  std::copy(t.Dth.begin(), t.Dth.end(), Dth);
  std::copy(t.Dph.begin(), t.Dph.end(), Dph);
  std::copy(t.Dvf.begin(), t.Dvf.end(), Dvf);
  return MF_OK;
}
