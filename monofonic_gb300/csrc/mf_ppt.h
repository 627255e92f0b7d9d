// Semiclassical (PPT) Eulerian fields of a species (ic_generator.cc:679-791).
#pragma once

#include "mf_runtime.h"

namespace mf {

struct PPTArgs {
  int n;
  double L;
  const void* f0;       // k-space phi(1), unscaled, grid precision
  const void* f1;       // k-space phi(2) or nullptr below 2LPT
  double g1, g2;        // growth factors of phi(1), phi(2) (ic_generator.cc:224-225)
  const void* delta_k;  // k-space delta_bc of the species (no relative-velocity amplitude) or nullptr
  void* delta_r;        // grid-precision padded real scratch for delta_bc
  double C;             // C_species
  double D, vunit;      // D+(a_start), D+ vfac / L * velocity_unit
  double* phi_r;        // two FP64 padded real scratch grids
  double* phi2_r;
  double2* psi;         // n^3 complex FP64
  double2* grad;        // 2 n^3 complex FP64
  double* maxd;         // device scalar
  double* rho_out;      // n^3 doubles: |psi|^2 - 1
  double* vel_out;      // 3 n^3 doubles
};

// 3D complex-to-complex transform of an n^3 FP64 field in place (unitary)
cudaError_t fft3d_c2c_f64(mf_ctx* c, double2* data, int n, bool inverse);
template <typename T>
cudaError_t ppt_eulerian(mf_ctx* c, const PPTArgs& a);

}  // namespace mf
