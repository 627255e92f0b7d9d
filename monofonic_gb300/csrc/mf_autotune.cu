// Autotuner of the convolution passes: per pass kind, transform length and
// precision it times the candidate schedules on a scratch convolution of the
// caller's grid size and keeps the fastest in a process-wide table that the
// launchers read (mf_sched.h).
//
// Candidates: the fused z pass as the TMA-pipelined kernel (radix-8 plan with
// radix-6/12 stages) with 1, 2 or the occupancy limit of persistent CTAs per
// SM, or as the direct-load kernel (radix-4 plan); the four strided passes
// with 1, 2 or the occupancy limit of persistent CTAs per SM.  A schedule
// changes which CTA processes which tile, not the arithmetic, except for the
// z-pass plan (radix-8 vs radix-4), which changes the rounding within the
// precision's tolerance.
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/monofonic_gb300.h"
#include "../../include/monofonic_gb300_ic.h"
#include "mf_runtime.h"
#include "mf_sched.h"

namespace mf {

namespace {
std::mutex g_mu;
std::map<std::tuple<int, int, int>, PassSched> g_table;
}  // namespace

PassSched sched_get(int kind, int L, int prec_bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(std::make_tuple(kind, L, prec_bytes));
  return it == g_table.end() ? PassSched{} : it->second;
}

void sched_set(int kind, int L, int prec_bytes, PassSched s) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[std::make_tuple(kind, L, prec_bytes)] = s;
}

void sched_clear() {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table.clear();
}

}  // namespace mf

using namespace mf;

namespace {

const char* kKindName[KK_COUNT] = {"conv_xinv", "conv_yinv", "conv_z", "conv_yfwd", "conv_xfwd",
                                   "fft_z", "fft_col", "pointwise"};

// device ms of one pass kind per convolve2, median of `reps` convolutions
int time_kind(mf_ctx* c, mf_conv* cv, mf_operand* a, mf_operand* b, mf_grid* out, int kind, int reps, double* ms) {
  std::vector<double> t;
  for (int r = 0; r < reps + 1; ++r) {
    mf_ctx_profile(c, 1);
    int rc = mf_conv_convolve2(cv, a, b, out, MF_OP_ASSIGN, 1.0);
    double acc[KK_COUNT];
    int64_t cnt[KK_COUNT];
    const int rc2 = mf_ctx_profile_read(c, acc, cnt, KK_COUNT);
    mf_ctx_profile(c, 0);
    if (rc != MF_OK) return rc;
    if (rc2 != MF_OK) return rc2;
    if (r > 0) t.push_back(acc[kind]);  // the first run warms the caches and the schedule
  }
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return MF_OK;
}

}  // namespace

extern "C" int mf_autotune(mf_ctx* c, int n, int prec, char* report, size_t report_len) {
  if (!c) return MF_ERR_ARG;
  if (!mf_grid_size_supported(n)) return set_err(c, MF_ERR_SHAPE, "mf_autotune: unsupported grid size");
  if (prec != MF_PREC_F32 && prec != MF_PREC_F64) return set_err(c, MF_ERR_ARG, "mf_autotune: bad precision");
  const int M = 3 * n / 2;
  const int pb = (prec == MF_PREC_F32) ? 4 : 8;
  mf_grid* f = nullptr;
  mf_grid* out = nullptr;
  mf_conv* cv = nullptr;
  int rc = mf_grid_create(c, n, 1.0, prec, MF_SPACE_R, &f);
  if (rc == MF_OK) rc = mf_grid_create(c, n, 1.0, prec, MF_SPACE_K, &out);
  if (rc == MF_OK) rc = mf_conv_create(c, n, 1.0, prec, MF_CONV_ORSZAG, &cv);
  if (rc == MF_OK) rc = mf_grid_fill_white_noise(f, 1234567);
  if (rc == MF_OK) rc = mf_grid_fft_forward(f, 1);
  std::string rep;
  if (rc == MF_OK) {
    mf_operand a{}, b{};
    a.grid = f;
    a.kind = MF_OPND_HESS;
    a.d[0] = 0; a.d[1] = 1;
    b.grid = f;
    b.kind = MF_OPND_SUM;
    b.d[0] = 1; b.d[1] = 1; b.d[2] = 2; b.d[3] = 2;
    const int reps = 3;
    const int kinds[5] = {KK_CONV_XINV, KK_CONV_YINV, KK_CONV_Z, KK_CONV_YFWD, KK_CONV_XFWD};
    for (int kind : kinds) {
      std::vector<PassSched> cand = {PassSched{0, 0}, PassSched{1, 0}, PassSched{2, 0}};
      if (kind == KK_CONV_Z) cand.push_back(PassSched{0, 1});
      PassSched best{};
      double best_ms = 1e30;
      char buf[256];
      std::snprintf(buf, sizeof buf, "%s L=%d %s:", kKindName[kind], M, pb == 4 ? "f32" : "f64");
      rep += buf;
      for (const PassSched& sc : cand) {
        sched_set(kind, M, pb, sc);
        double ms = 0;
        rc = time_kind(c, cv, &a, &b, out, kind, reps, &ms);
        if (rc != MF_OK) break;
        std::snprintf(buf, sizeof buf, " [occ %d%s %.4f ms]", sc.occ, sc.variant ? " direct" : "", ms);
        rep += buf;
        if (ms < best_ms) { best_ms = ms; best = sc; }
      }
      sched_set(kind, M, pb, best);
      if (rc != MF_OK) break;
      std::snprintf(buf, sizeof buf, " -> occ %d%s\n", best.occ, best.variant ? " direct" : "");
      rep += buf;
    }
  }
  if (cv) mf_conv_destroy(cv);
  if (out) mf_grid_destroy(out);
  if (f) mf_grid_destroy(f);
  if (report && report_len) {
    std::snprintf(report, report_len, "%s", rep.c_str());
  }
  return rc;
}

extern "C" int mf_autotune_reset(void) {
  sched_clear();
  return MF_OK;
}

extern "C" int mf_schedule_set(int kind, int L, int prec, int occ, int variant) {
  if (kind < KK_CONV_XINV || kind > KK_CONV_XFWD || L <= 0 || occ < 0 || variant < 0 || variant > 1) return MF_ERR_ARG;
  if (prec != MF_PREC_F32 && prec != MF_PREC_F64) return MF_ERR_ARG;
  if (variant == 1 && kind != KK_CONV_Z) return MF_ERR_ARG;
  sched_set(kind, L, prec == MF_PREC_F32 ? 4 : 8, PassSched{occ, variant});
  return MF_OK;
}
