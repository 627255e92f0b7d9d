// Recorded batch: many realizations (own grid size, seed and cosmology each)
// on one GPU as one CUDA graph launch.  Every realization owns a device
// pipeline (mf_ic); realizations are spread over a few streams, each stream
// runs its realizations back to back, and the streams overlap.  The graph
// is recorded once; a new seed or cosmology only changes the pipelines'
// parameter blocks, which the graph copies to the device when it runs.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/monofonic_gb300_batch.h"
#include "mf_request.h"
#include "mf_runtime.h"

using namespace mf;

struct mf_batch {
  int device = 0;
  std::vector<mf_ctx*> ctx;  // one context (stream) per lane
  cudaStream_t origin = nullptr;
  std::vector<mf_ic_request> items;
  std::vector<mf_ic*> ic;
  std::vector<int> lane;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> join;
  size_t device_bytes = 0;
  long long kernels = 0;
  std::string err;
  std::string tuning;  // autotuner report
};

namespace {

thread_local std::string g_create_err;  // message of a failed mf_batch_create on this thread

int berr(mf_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

int bcuda(mf_batch* b, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return MF_OK;
  return berr(b, e == cudaErrorMemoryAllocation ? MF_ERR_OOM : MF_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// cosmology scalars of items [first, first+count) on host threads
int compute_scalars(const mf_ic_request* items, int count, std::vector<mf_cosmo_scalars>& out, int nthreads) {
  out.assign(count, mf_cosmo_scalars{});
  std::vector<int> rc(count, MF_OK);
  parallel_for(count, nthreads, [&](int i) { rc[i] = mf_cosmology_compute(&items[i].cosmo, items[i].zstart, &out[i]); });
  for (int r : rc)
    if (r != MF_OK) return r;
  return MF_OK;
}

int record(mf_batch* b) {
  cudaError_t e;
  long long before = 0, after = 0;
  for (auto* c : b->ctx) {
    int64_t k[KK_COUNT] = {};
    mf_ctx_launch_counts(c, k, KK_COUNT);
    for (int64_t v : k) before += v;
  }
  if ((e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed)) != cudaSuccess)
    return bcuda(b, e, "begin capture");
  int rc = MF_OK;
  e = cudaEventRecord(b->fork, b->origin);
  for (size_t k = 0; e == cudaSuccess && k < b->ctx.size(); ++k) e = cudaStreamWaitEvent(b->ctx[k]->stream, b->fork, 0);
  if (e != cudaSuccess) rc = bcuda(b, e, "fork");
  for (size_t k = 0; rc == MF_OK && k < b->ctx.size(); ++k)
    for (size_t i = 0; rc == MF_OK && i < b->ic.size(); ++i)
      if (b->lane[i] == (int)k) {
        rc = mf_ic_enqueue(b->ic[i]);
        if (rc != MF_OK) berr(b, rc, std::string("record: ") + mf_last_error(b->ctx[k]));
      }
  for (size_t k = 0; rc == MF_OK && k < b->ctx.size(); ++k) {
    e = cudaEventRecord(b->join[k], b->ctx[k]->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->origin, b->join[k], 0);
    if (e != cudaSuccess) rc = bcuda(b, e, "join");
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(b->origin, &g);
  if (rc != MF_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bcuda(b, e, "end capture");
  b->graph = g;
  if ((e = cudaGraphInstantiate(&b->exec, g, 0)) != cudaSuccess) return bcuda(b, e, "graph instantiate");
  if ((e = cudaGraphUpload(b->exec, b->origin)) != cudaSuccess) return bcuda(b, e, "graph upload");
  if ((e = cudaStreamSynchronize(b->origin)) != cudaSuccess) return bcuda(b, e, "graph upload");
  for (auto* c : b->ctx) {
    int64_t k[KK_COUNT] = {};
    mf_ctx_launch_counts(c, k, KK_COUNT);
    for (int64_t v : k) after += v;
  }
  b->kernels = after - before;
  return MF_OK;
}

}  // namespace

extern "C" int mf_batch_destroy(mf_batch* b) {
  if (!b) return MF_ERR_ARG;
  cudaSetDevice(b->device);
  if (b->origin) cudaStreamSynchronize(b->origin);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto* p : b->ic)
    if (p) mf_ic_destroy(p);
  for (auto* c : b->ctx)
    if (c) mf_ctx_destroy(c);
  for (auto ev : b->join)
    if (ev) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return MF_OK;
}

extern "C" int mf_batch_create(int device, const mf_ic_request* items, int nitems, int nstreams, int flags,
                               mf_batch** out) {
  if (!out || !items || nitems <= 0) return MF_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < nitems; ++i) {
    const int rc = check_request(items[i]);
    if (rc != MF_OK) return rc;
  }
  if (nstreams <= 0) nstreams = 8;
  nstreams = std::min(nstreams, nitems);
  if (cudaSetDevice(device) != cudaSuccess) return MF_ERR_CUDA;
  mf_batch* b = new (std::nothrow) mf_batch();
  if (!b) return MF_ERR_OOM;
  b->device = device;
  b->items.assign(items, items + nitems);
  auto fail = [&](int rc) {
    // keep the message for the caller: it cannot reach a destroyed handle
    g_create_err = b->err.empty() ? std::string("mf_batch_create failed with status ") + std::to_string(rc) : b->err;
    mf_batch_destroy(b);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess) return fail(MF_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess)
    return fail(MF_ERR_CUDA);
  b->ctx.assign(nstreams, nullptr);
  b->join.assign(nstreams, nullptr);
  for (int k = 0; k < nstreams; ++k) {
    int rc = mf_ctx_create(device, &b->ctx[k]);
    if (rc != MF_OK) return fail(rc);
    if (cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming) != cudaSuccess) return fail(MF_ERR_CUDA);
  }
  std::vector<mf_cosmo_scalars> sc;
  int rc = compute_scalars(items, nitems, sc, 0);
  if (rc != MF_OK) return fail(rc);
  if (flags & MF_BATCH_AUTOTUNE) {  // schedules are read at launch, so tune before recording
    std::vector<std::pair<int, int>> shapes;
    for (int i = 0; i < nitems; ++i) {
      const std::pair<int, int> k(items[i].ngrid, items[i].precision);
      if (items[i].lpt_order > 1 && std::find(shapes.begin(), shapes.end(), k) == shapes.end()) shapes.push_back(k);
    }
    std::vector<char> rep(8192);
    for (const auto& k : shapes) {
      rc = mf_autotune(b->ctx[0], k.first, k.second, rep.data(), rep.size());
      if (rc != MF_OK) {
        b->err = std::string("autotune: ") + mf_last_error(b->ctx[0]);
        return fail(rc);
      }
      b->tuning += rep.data();
    }
  }
  // largest realization first onto the least loaded lane
  std::vector<int> order(nitems);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return request_cost(items[a]) > request_cost(items[c]); });
  std::vector<double> load(nstreams, 0.0);
  b->lane.assign(nitems, 0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    b->lane[i] = k;
    load[k] += request_cost(items[i]);
  }
  b->ic.assign(nitems, nullptr);
  for (int i = 0; i < nitems; ++i) {
    const mf_ic_params p = request_params(items[i], sc[i]);
    size_t fp = 0;
    mf_ic_device_footprint(&p, &fp);
    b->device_bytes += fp;
    rc = mf_ic_create(b->ctx[b->lane[i]], &p, &b->ic[i]);
    if (rc != MF_OK) {
      b->err = std::string("realization ") + std::to_string(i) + ": " + mf_last_error(b->ctx[b->lane[i]]);
      return fail(rc);
    }
    mf_ic_set_noise_seed(b->ic[i], items[i].seed);
  }
  for (auto* c : b->ctx)
    if ((rc = mf_ctx_synchronize(c)) != MF_OK) return fail(rc);
  if ((rc = record(b)) != MF_OK) return fail(rc);
  *out = b;
  return MF_OK;
}

extern "C" int mf_batch_set_items(mf_batch* b, int first, int count, const mf_cosmo_params* cosmo,
                                  const uint64_t* seeds, int nthreads) {
  if (!b || first < 0 || count < 0 || first + count > (int)b->items.size()) return MF_ERR_ARG;
  if (count == 0) return MF_OK;
  std::vector<mf_ic_request> req(b->items.begin() + first, b->items.begin() + first + count);
  for (int i = 0; i < count; ++i) {
    if (cosmo) req[i].cosmo = cosmo[i];
    if (seeds) req[i].seed = seeds[i];
  }
  std::vector<mf_cosmo_scalars> sc;
  if (cosmo) {
    const int rc = compute_scalars(req.data(), count, sc, nthreads);
    if (rc != MF_OK) return berr(b, rc, "mf_batch_set_items: cosmology");
  }
  for (int i = 0; i < count; ++i) {
    mf_ic* p = b->ic[first + i];
    if (cosmo) {
      const int rc = mf_ic_set_cosmology(p, &sc[i]);
      if (rc != MF_OK) return berr(b, rc, "mf_batch_set_items: set cosmology");
    }
    if (seeds) mf_ic_set_noise_seed(p, seeds[i]);
    b->items[first + i] = req[i];
  }
  return MF_OK;
}

extern "C" int mf_batch_run(mf_batch* b, double* ms) {
  if (!b || !b->exec) return MF_ERR_ARG;
  cudaSetDevice(b->device);
  cudaError_t e = cudaEventRecord(b->t0, b->origin);
  if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, b->origin);
  if (e == cudaSuccess) e = cudaEventRecord(b->t1, b->origin);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->origin);
  if (e != cudaSuccess) return bcuda(b, e, "mf_batch_run");
  for (auto* c : b->ctx) {
    const int rc = mf_ctx_synchronize(c);  // raised device error flags (bounded waits)
    if (rc != MF_OK) return berr(b, rc, std::string("mf_batch_run: ") + mf_last_error(c));
  }
  if (ms) {
    float t = 0;
    cudaEventElapsedTime(&t, b->t0, b->t1);
    *ms = t;
  }
  return MF_OK;
}

extern "C" int mf_batch_particles(mf_batch* b, int i, mf_particles* out) {
  if (!b || !out || i < 0 || i >= (int)b->ic.size()) return MF_ERR_ARG;
  return mf_ic_particles(b->ic[i], out);
}

extern "C" int mf_batch_info(mf_batch* b, int* graph_nodes, long long* kernels, size_t* device_bytes) {
  if (!b) return MF_ERR_ARG;
  if (graph_nodes) {
    size_t n = 0;
    if (b->graph) cudaGraphGetNodes(b->graph, nullptr, &n);
    *graph_nodes = (int)n;
  }
  if (kernels) *kernels = b->kernels;
  if (device_bytes) *device_bytes = b->device_bytes;
  return MF_OK;
}

extern "C" const char* mf_batch_tuning(const mf_batch* b) { return b ? b->tuning.c_str() : ""; }

extern "C" const char* mf_batch_last_error(const mf_batch* b) { return b ? b->err.c_str() : g_create_err.c_str(); }
