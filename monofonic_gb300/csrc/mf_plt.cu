// PLT tables: lattice_gradient::init_D (include/particle_plt.hh:68-515) on the
// device.  Four steps, each a kernel over the ng^3 PLT mesh (or its ng^2
// (ng/2+1) modes): Ewald sums of the dynamical matrix per cell, the r2c
// transforms of its six components, the 3x3 eigen-decomposition with the
// first-Brillouin-zone mapping, and the neighbour averaging with the
// projection onto spherical unit vectors.  The reference's std::map from FBZ
// mesh index to mode (insert keeps the first mode in loop order) becomes a
// dense index box filled with atomicMin of the loop position.
#include <algorithm>
#include <array>
#include <climits>
#include <initializer_list>
#include <cmath>
#include <vector>

#include "../../include/monofonic_gb300_ic.h"
#include "mf_plt.h"

namespace mf {
namespace {

constexpr int kFBZCand = 54;  // l1, l2, l3 in -1..1, two signs (particle_plt.hh:358-380)

struct PLTLattice {
  double B[9], R[9];  // Bravais and reciprocal matrices, row-major
  int IR[9];          // inverse reciprocal matrix
  double normals[14][3];
  int nnormals;
  int charge_fac;
};

// Bravais, reciprocal and inverse-reciprocal matrices and FBZ normals
// (particle_plt.hh:76-164); RSC uses the SC set as in the reference
PLTLattice lattice_set(int lattice) {
  const double pi = M_PI, twopi = 2 * M_PI, fourpi = 4 * M_PI;
  PLTLattice L{};
  auto setv = [](double* d, std::initializer_list<double> v) { std::copy(v.begin(), v.end(), d); };
  auto seti = [](int* d, std::initializer_list<int> v) { std::copy(v.begin(), v.end(), d); };
  std::vector<std::array<double, 3>> nrm;
  if (lattice == MF_LATTICE_BCC) {
    L.charge_fac = 2;
    setv(L.B, {1, 0, 0.5, 0, 1, 0.5, 0, 0, 0.5});
    setv(L.R, {twopi, 0, 0, 0, twopi, 0, -twopi, -twopi, fourpi});
    seti(L.IR, {2, 0, 0, 0, 2, 0, 1, 1, 1});
    nrm = {{0, pi, pi},  {0, -pi, pi},  {0, pi, -pi},  {0, -pi, -pi}, {pi, 0, pi},  {-pi, 0, pi},
           {pi, 0, -pi}, {-pi, 0, -pi}, {pi, pi, 0},   {-pi, pi, 0},  {pi, -pi, 0}, {-pi, -pi, 0}};
  } else if (lattice == MF_LATTICE_FCC) {
    L.charge_fac = 4;
    setv(L.B, {0, 0.5, 0, 0.5, 0, 1, 0.5, 0.5, 0});
    setv(L.R, {-fourpi, fourpi, twopi, 0, 0, twopi, fourpi, 0, -twopi});
    seti(L.IR, {0, 1, 1, 1, 0, 1, 0, 2, 0});
    nrm = {{twopi, 0, 0}, {-twopi, 0, 0}, {0, twopi, 0},  {0, -twopi, 0}, {0, 0, twopi},  {0, 0, -twopi},
           {pi, pi, pi},  {pi, pi, -pi},  {pi, -pi, pi},  {pi, -pi, -pi}, {-pi, pi, pi},  {-pi, pi, -pi},
           {-pi, -pi, pi}, {-pi, -pi, -pi}};
  } else {
    L.charge_fac = 1;
    setv(L.B, {1, 0, 0, 0, 1, 0, 0, 0, 1});
    setv(L.R, {twopi, 0, 0, 0, twopi, 0, 0, 0, twopi});
    seti(L.IR, {2, 0, 0, 0, 2, 0, 0, 0, 2});
    nrm = {{pi, 0, 0}, {-pi, 0, 0}, {0, pi, 0}, {0, -pi, 0}, {0, 0, pi}, {0, 0, -pi}};
  }
  L.nnormals = (int)nrm.size();
  for (int a = 0; a < L.nnormals; ++a)
    for (int b = 0; b < 3; ++b) L.normals[a][b] = nrm[a][b];
  return L;
}

__device__ __forceinline__ void mat_vec(const double* A, double x, double y, double z, double* o) {
  o[0] = A[0] * x + A[1] * y + A[2] * z;
  o[1] = A[3] * x + A[4] * y + A[5] * z;
  o[2] = A[6] * x + A[7] * y + A[8] * z;
}

// ---- 1. Ewald sums of the dynamical matrix in real space (particle_plt.hh:167-269)
// One thread per mesh cell; the six independent components go to six padded
// real grids (row stride nl+2) for the transforms.
struct EwaldArgs {
  PLTLattice L;
  int nl;
  double alpha, alpha2, alpha3, charge, fft_norm;
  double sqrtpi, pi32;  // sqrt(pi) and pi^1.5 of the double pi, as the host computes them
  double* D6[6];
};

__global__ void __launch_bounds__(128) k_plt_ewald(EwaldArgs a) {
  const int nl = a.nl;
  const size_t n3 = (size_t)nl * nl * nl;
  const size_t cell = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (cell >= n3) return;
  const int i = (int)(cell / ((size_t)nl * nl)), j = (int)((cell / nl) % nl), k = (int)(cell % nl);
  const double dx = 1.0 / nl;
  const double pi32 = a.pi32, sqrtpi = a.sqrtpi;
  const double fourpi = 4 * M_PI;
  double ar[3];
  mat_vec(a.L.B, dx * i, dx * j, dx * k, ar);
  for (int d = 0; d < 3; ++d) ar[d] = fmod(2.0 + ar[d], 1.0);  // wrap_abs (vec3.hh:111-114)
  double M[6] = {0, 0, 0, 0, 0, 0};  // xx xy xz yy yz zz
  for (int ix = -3; ix <= 3; ++ix)
    for (int iy = -3; iy <= 3; ++iy)
      for (int iz = -3; iz <= 3; ++iz) {
        double bn[3];
        mat_vec(a.L.B, (double)ix, (double)iy, (double)iz, bn);
        const double d0 = ar[0] - bn[0], d1 = ar[1] - bn[1], d2 = ar[2] - bn[2];
        const double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        if (r < 1e-14) continue;
        const double r2 = r * r, r3 = r2 * r, r5 = r3 * r2;
        const double ex = exp(-a.alpha2 * r2);
        const double K1 = -a.alpha3 / pi32 * ex / r2;
        const double K2 = (erfc(a.alpha * r) + 2.0 * a.alpha / sqrtpi * ex * r) / fourpi;
        const double dv[3] = {d0, d1, d2};
        int m = 0;
        for (int mu = 0; mu < 3; ++mu)
          for (int nu = mu; nu < 3; ++nu, ++m)
            M[m] += dv[mu] * dv[nu] * K1 + ((mu == nu ? 1.0 : 0.0) / r3 - 3.0 * (dv[mu] * dv[nu]) / r5) * K2;
      }
  for (int ix = -3; ix <= 3; ++ix)
    for (int iy = -3; iy <= 3; ++iy)
      for (int iz = -3; iz <= 3; ++iz) {
        if (abs(ix) + abs(iy) + abs(iz) == 0) continue;
        double ak[3];
        mat_vec(a.L.R, (double)ix / nl, (double)iy / nl, (double)iz / nl, ak);
        const double kmod2 = ak[0] * ak[0] + ak[1] * ak[1] + ak[2] * ak[2];
        const double term =
            exp(-kmod2 / (4 * a.alpha2)) * cos(ak[0] * ar[0] + ak[1] * ar[1] + ak[2] * ar[2]) / kmod2 * a.fft_norm;
        int m = 0;
        for (int mu = 0; mu < 3; ++mu)
          for (int nu = mu; nu < 3; ++nu, ++m) M[m] += ak[mu] * ak[nu] * term;
      }
  const size_t o = ((size_t)i * nl + j) * (nl + 2) + k;
  if (cell == 0) {  // r = 0 with the background density (particle_plt.hh:263-269)
    const double v0[6] = {1.0 / 3.0, 0.0, 0.0, 1.0 / 3.0, 0.0, 1.0 / 3.0};
    for (int m = 0; m < 6; ++m) a.D6[m][o] = v0[m];
  } else {
    for (int m = 0; m < 6; ++m) a.D6[m][o] = M[m] * a.charge;
  }
}

// cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix; eigenvalues
// ascending (as gsl_eigen_symmv + GSL_EIGEN_SORT_VAL_ASC, mat3.hh:169-190),
// eigenvectors as columns of V
__device__ void eigen3(double* A, double* ev, double* V) {
  for (int q = 0; q < 9; ++q) V[q] = (q % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    if (off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const double apq = A[3 * p + q];
        if (apq == 0.0) continue;
        const double app = A[3 * p + p], aqq = A[3 * q + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
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
  int idx[3] = {0, 1, 2};
  const double e[3] = {A[0], A[4], A[8]};
  for (int x = 1; x < 3; ++x)  // insertion sort by eigenvalue, ascending
    for (int y = x; y > 0 && e[idx[y]] < e[idx[y - 1]]; --y) {
      const int t = idx[y];
      idx[y] = idx[y - 1];
      idx[y - 1] = t;
    }
  double V0[9];
  for (int q = 0; q < 9; ++q) V0[q] = V[q];
  for (int c2 = 0; c2 < 3; ++c2) {
    ev[c2] = e[idx[c2]];
    for (int r = 0; r < 3; ++r) V[3 * r + c2] = V0[3 * r + idx[c2]];
  }
}

// dense box of FBZ mesh indices: each coordinate in [-ng-1, ng+1]
struct FBZMap {
  unsigned long long* slot;
  int ng, side;
  __device__ __forceinline__ long long key(int ix, int iy, int iz) const {
    const int o = ng + 1;
    if (ix < -o || ix > o || iy < -o || iy > o || iz < -o || iz > o) return -1;
    return ((long long)(ix + o) * side + (iy + o)) * side + (iz + o);
  }
};

// ---- 2. eigen-decomposition and first-Brillouin-zone mapping (particle_plt.hh:295-390)
// T6: [6][nkt] = (T1r, T1i, T2r, T2i, T3r, T3i); slot value = mode * 54 + candidate
struct EigenArgs {
  PLTLattice L;
  int nl, ng;
  double fft_norm12;
  const double* Dk[6];  // padded complex grids after the r2c (real part at 2q)
  double* T6;
  FBZMap map;
  int* err;
};

__global__ void __launch_bounds__(128) k_plt_eigen_fbz(EigenArgs a) {
  const int nl = a.nl, nk = nl / 2 + 1;
  const size_t nkt = (size_t)nl * nl * nk;
  const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= nkt) return;
  const int i = (int)(q / ((size_t)nl * nk)), j = (int)((q / nk) % nl), k = (int)(q % nk);
  const double twopi = 2 * M_PI;
  auto kcomp = [&](int idx) { return (double(idx) - double(idx > nl / 2) * nl) * twopi; };
  double dk[6];
  for (int m = 0; m < 6; ++m) dk[m] = a.Dk[m][2 * q];
  double T[6] = {dk[0], dk[1], dk[2], dk[3], dk[4], dk[5]};
  double D[9] = {dk[0] / a.fft_norm12, dk[1] / a.fft_norm12, dk[2] / a.fft_norm12,
                 dk[1] / a.fft_norm12, dk[3] / a.fft_norm12, dk[4] / a.fft_norm12,
                 dk[2] / a.fft_norm12, dk[4] / a.fft_norm12, dk[5] / a.fft_norm12};
  double ev[3], Vm[9];
  eigen3(D, ev, Vm);
  const double tn = twopi * a.ng;
  const double e3[3] = {Vm[2] / tn, Vm[5] / tn, Vm[8] / tn};
  double av[3];
  mat_vec(a.L.R, kcomp(i) / tn, kcomp(j) / tn, kcomp(k) / tn, av);
  int cand = 0;
  for (int l1 = -1; l1 <= 1; ++l1)
    for (int l2 = -1; l2 <= 1; ++l2)
      for (int l3 = -1; l3 <= 1; ++l3)
        for (int is = 0; is <= 1; ++is, ++cand) {
          const double sg = 2.0 * is - 1.0;
          double rs[3];
          mat_vec(a.L.R, (double)l1, (double)l2, (double)l3, rs);
          const double vk[3] = {sg * av[0] + rs[0], sg * av[1] + rs[1], sg * av[2] + rs[2]};
          bool in = true;
          for (int nn = 0; nn < a.L.nnormals; ++nn) {
            const double* nr = a.L.normals[nn];
            if (nr[0] * vk[0] + nr[1] * vk[1] + nr[2] * vk[2] > 1.0001 * (nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]))
              in = false;
          }
          if (!in) continue;
          const int ix = (int)round(vk[0] * a.ng / twopi);
          const int iy = (int)round(vk[1] * a.ng / twopi);
          const int iz = (int)round(vk[2] * a.ng / twopi);
          const long long key = a.map.key(ix, iy, iz);
          if (key < 0) {
            atomicExch(a.err, 1);
            continue;
          }
          atomicMin(&a.map.slot[key], (unsigned long long)q * kFBZCand + cand);
          T[0] = ev[2]; T[1] = ev[1];
          T[2] = ev[0]; T[3] = e3[0];
          T[4] = e3[1]; T[5] = e3[2];
        }
  for (int m = 0; m < 6; ++m) a.T6[(size_t)m * nkt + q] = T[m];
}

// ---- 3. neighbour averaging onto the regular mesh (particle_plt.hh:401-458) and
// projection onto spherical unit vectors (:461-487); out: Dr, Dth, Dph, Dvf [4][nkt]
struct ProjectArgs {
  int IR[9];
  int nl;
  const double* T6;
  FBZMap map;
  double* out;
};

__global__ void __launch_bounds__(128) k_plt_project(ProjectArgs a) {
  const int nl = a.nl, nk = nl / 2 + 1;
  const size_t nkt = (size_t)nl * nl * nk;
  const size_t q0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q0 >= nkt) return;
  const int i = (int)(q0 / ((size_t)nl * nk)), j = (int)((q0 / nk) % nl), k = (int)(q0 % nk);
  const int ii = (i > nl / 2) ? i - nl : i, jj = (j > nl / 2) ? j - nl : j, kk = (k > nl / 2) ? k - nl : k;
  const double* T = a.T6;
  auto lookup = [&](int x, int y, int z) -> long long {
    const long long key = a.map.key(x, y, z);
    if (key < 0) return -1;
    const unsigned long long v = a.map.slot[key];
    return v == ULLONG_MAX ? -1 : (long long)(v / kFBZCand);
  };
  auto align = [&](double* v) {  // sign of the eigenvector along the mode
    if (v[0] * ii + v[1] * jj + v[2] * kk < 0.0)
      for (int d = 0; d < 3; ++d) v[d] = -v[d];
  };
  bool in = true;
  for (int r = 0; r < 3; ++r)
    if ((a.IR[3 * r] * i + a.IR[3 * r + 1] * j + a.IR[3 * r + 2] * k) % 2 != 0) in = false;
  double l[3] = {0, 0, 0}, v[3] = {0, 0, 0};
  if (!in) {
    int count = 0;
    const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    for (int o = 0; o < 6; ++o) {
      const long long q = lookup(ii + nb[o][0], jj + nb[o][1], kk + nb[o][2]);
      if (q < 0) continue;
      ++count;
      l[0] += T[q]; l[1] += T[nkt + q]; l[2] += T[2 * nkt + q];
      double e[3] = {T[3 * nkt + q], T[4 * nkt + q], T[5 * nkt + q]};
      align(e);
      v[0] += e[0]; v[1] += e[1]; v[2] += e[2];
    }
    for (int d = 0; d < 3; ++d) {
      l[d] /= double(count);
      v[d] /= double(count);
    }
  } else {
    const long long q = lookup(ii, jj, kk);
    if (q >= 0) {
      l[0] = T[q]; l[1] = T[nkt + q]; l[2] = T[2 * nkt + q];
      v[0] = T[3 * nkt + q]; v[1] = T[4 * nkt + q]; v[2] = T[5 * nkt + q];
      align(v);
    }
  }
  const double twopi = 2 * M_PI;
  auto kcomp = [&](int idx) { return (double(idx) - double(idx > nl / 2) * nl) * twopi; };
  const double kv[3] = {kcomp(i), kcomp(j), kcomp(k)};
  const double mu1 = l[0];
  double e1[3] = {v[0], v[1], v[2]};
  const double en = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
  for (int d = 0; d < 3; ++d) e1[d] /= en;
  const double kr = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
  const double kphi = kr > 0.0 ? atan2(kv[1], kv[0]) : 0.0;
  const double kth = kr > 0.0 ? acos(kv[2] / kr) : 0.0;
  const double st = sin(kth), ct = cos(kth), sp = sin(kphi), cp = cos(kphi);
  const double e_r[3] = {st * cp, st * sp, ct}, e_t[3] = {ct * cp, ct * sp, -st}, e_p[3] = {-sp, cp, 0.0};
  double renorm = e1[0] * e_r[0] + e1[1] * e_r[1] + e1[2] * e_r[2];
  if (renorm < 0.01) renorm = 1.0;
  double Dr = 1.0, Dth = (e1[0] * e_t[0] + e1[1] * e_t[1] + e1[2] * e_t[2]) / renorm,
         Dph = (e1[0] * e_p[0] + e1[1] * e_p[1] + e1[2] * e_p[2]) / renorm,
         Dvf = 1.0 / (0.25 * (sqrt(1. + 24 * mu1) - 1.));
  if (q0 == 0) {
    Dr = 1.0; Dth = 0.0; Dph = 0.0; Dvf = 1.0;
  }
  a.out[q0] = Dr;
  a.out[nkt + q0] = Dth;
  a.out[2 * nkt + q0] = Dph;
  a.out[3 * nkt + q0] = Dvf;
}

unsigned blocks128(size_t n) { return (unsigned)((n + 127) / 128); }

}  // namespace

int plt_build_tables(mf_ctx* c, int lattice, int ng, PLTTables* out) {
  if (!grid_size_supported(ng)) return set_err(c, MF_ERR_SHAPE, "PLT mesh size not supported");
  cudaStream_t s = c->stream;
  const PLTLattice LT = lattice_set(lattice);
  const int nl = ng, nk = nl / 2 + 1;
  const size_t nkt = (size_t)nl * nl * nk, n3 = (size_t)nl * nl * nl;
  const size_t greals = grid_reals(nl);
  const int side = 2 * ng + 3;
  const size_t nslots = (size_t)side * side * side;
  // one allocation: six padded grids, T6, the four tables, the FBZ map, the error flag
  const size_t bytes = (6 * greals + 6 * nkt + 4 * nkt) * sizeof(double) + nslots * sizeof(unsigned long long) + 16;
  char* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, bytes, s);
  if (e != cudaSuccess) return cuda_err(c, e, "PLT: device buffers");
  double* grids = reinterpret_cast<double*>(buf);
  double* T6 = grids + 6 * greals;
  double* tabs = T6 + 6 * nkt;
  unsigned long long* slots = reinterpret_cast<unsigned long long*>(tabs + 4 * nkt);
  int* err = reinterpret_cast<int*>(slots + nslots);
  int herr = 0;
  std::vector<double> h(4 * nkt);
#define CK(x)                                    \
  do {                                           \
    e = (x);                                     \
    if (e != cudaSuccess) goto done;             \
  } while (0)
  {
    CK(cudaMemsetAsync(grids, 0, 6 * greals * sizeof(double), s));
    CK(cudaMemsetAsync(slots, 0xff, nslots * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(err, 0, sizeof(int), s));
    EwaldArgs ea{};
    ea.L = LT;
    ea.nl = nl;
    const double eta = 4.0;
    ea.alpha = 1.0 / std::sqrt(2.0) / eta;
    ea.alpha2 = ea.alpha * ea.alpha;
    ea.alpha3 = ea.alpha2 * ea.alpha;
    ea.charge = 1.0 / std::pow(double(nl), 3) / LT.charge_fac;
    ea.fft_norm = 1.0 / std::pow(double(nl), 3.0);
    ea.sqrtpi = std::sqrt(M_PI);
    ea.pi32 = std::pow(M_PI, 1.5);
    for (int m = 0; m < 6; ++m) ea.D6[m] = grids + m * greals;
    {
      LaunchScope ls(c, KK_POINTWISE);
      k_plt_ewald<<<blocks128(n3), 128, 0, s>>>(ea);
      CK(cudaGetLastError());
    }
    // forward transforms (unitary), real parts read by the eigen pass
    for (int m = 0; m < 6; ++m) CK(fft3d_r2c<double>(c, grids + m * greals, nl));
    EigenArgs ga{};
    ga.L = LT;
    ga.nl = nl;
    ga.ng = ng;
    ga.fft_norm12 = 1.0 / std::pow(double(nl), 1.5);
    for (int m = 0; m < 6; ++m) ga.Dk[m] = grids + m * greals;
    ga.T6 = T6;
    ga.map = FBZMap{slots, ng, side};
    ga.err = err;
    {
      LaunchScope ls(c, KK_POINTWISE);
      k_plt_eigen_fbz<<<blocks128(nkt), 128, 0, s>>>(ga);
      CK(cudaGetLastError());
    }
    ProjectArgs pa{};
    std::copy(LT.IR, LT.IR + 9, pa.IR);
    pa.nl = nl;
    pa.T6 = T6;
    pa.map = ga.map;
    pa.out = tabs;
    {
      LaunchScope ls(c, KK_POINTWISE);
      k_plt_project<<<blocks128(nkt), 128, 0, s>>>(pa);
      CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(h.data(), tabs, 4 * nkt * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
done:
#undef CK
  cudaFreeAsync(buf, s);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(s);
    return cuda_err(c, e, "PLT: init_D on the device");
  }
  if (herr) return set_err(c, MF_ERR_STATE, "PLT: FBZ mesh index outside the map");
  out->ng = ng;
  out->lattice = lattice;
  out->Dr.assign(h.begin(), h.begin() + nkt);
  out->Dth.assign(h.begin() + nkt, h.begin() + 2 * nkt);
  out->Dph.assign(h.begin() + 2 * nkt, h.begin() + 3 * nkt);
  out->Dvf.assign(h.begin() + 3 * nkt, h.end());
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
