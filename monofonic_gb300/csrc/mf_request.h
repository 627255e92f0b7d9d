// Shared host helpers of the batch and server front ends: one request ->
// pipeline parameters, a parallel loop over host threads.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "../../include/monofonic_gb300_batch.h"

namespace mf {

inline int check_request(const mf_ic_request& r) {
  if (r.lpt_order < 1 || r.lpt_order > 3) return MF_ERR_ARG;
  if (r.lattice < MF_LATTICE_SC || r.lattice > MF_LATTICE_RSC) return MF_ERR_ARG;
  if (r.precision != MF_PREC_F32 && r.precision != MF_PREC_F64) return MF_ERR_ARG;
  if (!(r.boxlen > 0) || !(r.zstart >= 0)) return MF_ERR_ARG;
  if (!mf_grid_size_supported(r.ngrid)) return MF_ERR_SHAPE;
  return MF_OK;
}

// pipeline parameters of a request (cosmology scalars passed in): Orszag
// convolver, particle output in box units (lunit = vunit = boxlen)
inline mf_ic_params request_params(const mf_ic_request& r, const mf_cosmo_scalars& sc) {
  mf_ic_params p{};
  p.ngrid = r.ngrid;
  p.boxlen = r.boxlen;
  p.zstart = r.zstart;
  p.lpt_order = r.lpt_order;
  p.lattice = r.lattice;
  p.precision = r.precision;
  p.convolver = MF_CONV_ORSZAG;
  p.cosmo = sc;
  p.tk_table = nullptr;
  p.lunit = r.boxlen;
  p.vunit = r.boxlen;
  p.out_kind = MF_OUT_PARTICLES;
  p.pos64 = r.pos64;
  p.id64 = r.id64;
  return p;
}

// relative device cost of a request (convolutions x padded volume x log)
inline double request_cost(const mf_ic_request& r) {
  const double n = r.ngrid, m = 1.5 * n;
  const double nconv = (r.lpt_order == 3) ? 33.0 : (r.lpt_order == 2 ? 5.0 : 0.0);
  const double f = (r.precision == MF_PREC_F64) ? 10.0 : 1.0;
  return f * ((nconv * 5.0) * m * m * m * std::log2(m) + (6.0 * (1 << r.lattice) + 3.0) * n * n * n * std::log2(n));
}

// f(i) for i in [0, n) on up to nthreads host threads (<= 0: all)
template <class F>
void parallel_for(int n, int nthreads, F f) {
  if (n <= 0) return;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  nthreads = std::min(nthreads, n);
  if (nthreads == 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([&] {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& t : th) t.join();
}

}  // namespace mf
