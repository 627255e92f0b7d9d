// Particle-linear-theory (PLT) corrected gradient and growth rate
// (Joyce & Marcos), restated from include/particle_plt.hh.
#pragma once

#include <cmath>
#include <vector>

#include "mf_plt_dev.cuh"
#include "mf_runtime.h"

namespace mf {

// tables on the ng^3 PLT mesh (built on the device, returned to the host), k-space layout [i][j][k], k <= ng/2
// (real parts of D_xx, D_yy, D_zz, D_xy after init_D, particle_plt.hh:461-487)
struct PLTTables {
  int ng = 0;
  int lattice = 0;
  std::vector<double> Dr, Dth, Dph, Dvf;
};

// init_D (particle_plt.hh:68-515): Ewald dynamical matrix on the ng^3 mesh,
// r2c, 3x3 eigen-decomposition, first-Brillouin-zone mapping,
// neighbour averaging, projection onto spherical unit vectors
int plt_build_tables(mf_ctx* c, int lattice, int ng, PLTTables* out);

}  // namespace mf
