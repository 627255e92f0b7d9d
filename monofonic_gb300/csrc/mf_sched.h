// Runtime schedules of the FFT pass kernels, chosen by the autotuner
// (mf_autotune) and read by the launchers at every launch.
#pragma once

namespace mf {

// schedule of one pass kind (KernelKind) at one transform length and
// precision; zero fields mean the compiled default
struct PassSched {
  int occ = 0;      // persistent kernels: CTAs per SM (capped by the occupancy limit)
  int variant = 0;  // fused z pass: 0 TMA-pipelined radix-8 plan, 1 direct-load radix-4 plan
};

PassSched sched_get(int kind, int L, int prec_bytes);
void sched_set(int kind, int L, int prec_bytes, PassSched s);
void sched_clear();

}  // namespace mf
