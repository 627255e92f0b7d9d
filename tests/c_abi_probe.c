/* A plain C99 client of libmfgpu: includes every public header and calls the
 * host-side entry points that need no GPU.  tests/test_cpu_c_abi.py compiles
 * it with -Werror and runs it. */
#include <stdio.h>
#include <string.h>

#include "monofonic_gb300.h"
#include "monofonic_gb300_batch.h"
#include "monofonic_gb300_ic.h"
#include "monofonic_gb300_output.h"

int main(void) {
  const char* v = mf_version();
  if (!v || !*v) return 1;
  if (mf_grid_size_supported(512) != 1 || mf_grid_size_supported(100) != 0) return 2;

  mf_cosmo_params cp;
  mf_cosmo_params_default(&cp); /* unset keys, then the configuration's */
  cp.Omega_b = 0.0488;
  cp.h = 0.6774;
  cp.n_s = 0.9667;
  mf_cosmo_scalars sc;
  if (mf_cosmology_compute(&cp, 24.0, &sc) != MF_OK) return 3;
  if (!(sc.Dplus > 0 && sc.Dplus < 1) || !(sc.pnorm > 0)) return 4;

  double k[3] = {1e-3, 0.1, 1.0}, t[3];
  if (mf_eh_transfer(&cp, k, t, 3) != MF_OK || !(t[0] > t[1] && t[1] > t[2] && t[2] > 0)) return 5;

  mf_ic_params p;
  memset(&p, 0, sizeof p);
  p.ngrid = 64;
  p.boxlen = 100.0;
  p.zstart = 24.0;
  p.lpt_order = 3;
  p.lattice = MF_LATTICE_BCC;
  p.precision = MF_PREC_F32;
  p.convolver = MF_CONV_ORSZAG;
  p.out_kind = MF_OUT_PARTICLES;
  p.cosmo = sc;
  p.pos64 = 1;
  p.id64 = 1;
  int64_t np = 0;
  size_t pb = 0, vb = 0, ib = 0, dev = 0;
  if (mf_ic_output_size(&p, &np, &pb, &vb, &ib) != MF_OK) return 6;
  if (np != 2 * 64 * 64 * 64 || pb != (size_t)np * 24 || ib != (size_t)np * 8) return 7;
  if (mf_ic_device_footprint(&p, &dev) != MF_OK || dev <= pb + vb + ib) return 8;
  p.ngrid = 100;
  if (mf_ic_output_size(&p, &np, &pb, &vb, &ib) != MF_ERR_SHAPE) return 9;

  double noise[8 * 8 * 8];
  if (mf_white_noise_host(8, 12345u, noise, 1) != MF_OK) return 10;
  printf("%s %.17g %.17g %.17g\n", v, sc.Dplus, sc.pnorm, noise[0]);
  return 0;
}
