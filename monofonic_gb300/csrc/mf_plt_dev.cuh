// Device-side evaluation of the PLT corrected gradient (include/particle_plt.hh:551-585).
#pragma once

#include <cmath>
#include <cstddef>

#include "mf_fft.cuh"

namespace mf {

// device copy of the tables in one precision
template <typename T>
struct PLTDev {
  const T* Dr = nullptr;
  const T* Dth = nullptr;
  const T* Dph = nullptr;
  const T* Dvf = nullptr;
  int ng = 0;
  T mapratio = 0;  // ng / N
  T inv_mr_L = 0;  // 1 / (mapratio * boxlen)
};

// get_cic_kspace (grid_fft.hh:347-373) of a real table: CIC weights in index
// space, periodic in i and j, clamped at the last kz plane
template <typename T>
__device__ __forceinline__ T plt_cic(const T* __restrict__ tab, int ng, T x, T y, T z) {
  const int nk = ng / 2 + 1;
  const int ix = (int)floor(x), iy = (int)floor(y), iz = (int)floor(z);
  const T dx = x - T(ix), tx = T(1) - dx;
  const T dy = y - T(iy), ty = T(1) - dy;
  const T dz = z - T(iz), tz = T(1) - dz;
  // x, y in [0, ng): the periodic neighbour wraps only at the last index
  const int ix1 = (ix + 1 == ng) ? 0 : ix + 1, iy1 = (iy + 1 == ng) ? 0 : iy + 1, iz1 = min(iz + 1, nk - 1);
  auto at = [&](int a, int b, int k) { return tab[((size_t)a * ng + b) * nk + k]; };
  T v = T(0);
  v += at(ix, iy, iz) * tx * ty * tz;
  v += at(ix, iy, iz1) * tx * ty * dz;
  v += at(ix, iy1, iz) * tx * dy * tz;
  v += at(ix, iy1, iz1) * tx * dy * dz;
  v += at(ix1, iy, iz) * dx * ty * tz;
  v += at(ix1, iy, iz1) * dx * ty * dz;
  v += at(ix1, iy1, iz) * dx * dy * tz;
  v += at(ix1, iy1, iz1) * dx * dy * dz;
  return v;
}

// lattice_gradient::gradient for all three directions and vfac_corr
// (particle_plt.hh:551-585) at N-grid mode (i, j, kz); returns the real
// factors g[d] of the purely imaginary gradient i*g[d].  The spherical unit
// vectors are formed from k directly (sin/cos of atan2/acos angles written
// as ratios of k components).
template <typename T>
__device__ __forceinline__ void plt_gradient(const PLTDev<T>& P, int i, int j, int kz, T g[3], T* vcorr) {
  const int ng = P.ng;
  const T x = T(i) * P.mapratio, y = T(j) * P.mapratio, z = T(kz) * P.mapratio;
  const T half = T(ng / 2), two_pi = T(6.283185307179586476925286766559);
  const T kx = (x - ((x > half) ? T(ng) : T(0))) * two_pi;
  const T ky = (y - ((y > half) ? T(ng) : T(0))) * two_pi;
  const T kz2 = (z - ((z > half) ? T(ng) : T(0))) * two_pi;
  const T kr = sqrt(kx * kx + ky * ky + kz2 * kz2);
  const T kmod = kr * P.inv_mr_L;
  const T Dr = plt_cic(P.Dr, ng, x, y, z), Dt = plt_cic(P.Dth, ng, x, y, z), Dp = plt_cic(P.Dph, ng, x, y, z);
  T st = T(0), ct = T(1), sp = T(0), cp = T(1);
  if (kr > T(0)) {
    const T kp = sqrt(kx * kx + ky * ky);
    const T ir = rcp_rn(kr);
    st = kp * ir;
    ct = kz2 * ir;
    if (kp > T(0)) {
      const T ip = rcp_rn(kp);
      sp = ky * ip;
      cp = kx * ip;
    }
  }
  g[0] = kmod * (Dr * st * cp + Dt * ct * cp - Dp * sp);
  g[1] = kmod * (Dr * st * sp + Dt * ct * sp + Dp * cp);
  g[2] = kmod * (Dr * ct - Dt * st);
  if (vcorr) *vcorr = plt_cic(P.Dvf, ng, x, y, z);
}

}  // namespace mf
