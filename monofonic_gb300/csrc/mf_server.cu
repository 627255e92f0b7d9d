// Continuous-batching IC server on one GPU.
//
// Requests wait in a FIFO queue.  nworkers host threads take requests as
// soon as one is admissible: a worker is free and the request's pipeline is
// either pooled idle (same grid, box, order, lattice, precision and output
// types) or fits the device-memory budget next to every live pipeline, after
// evicting idle pooled ones if needed.  Every pipeline has its own context
// and stream, so pipelines of different requests run concurrently on the
// device and any worker can drive any pooled pipeline.  A request waiting
// longer than the starvation limit stops later requests from overtaking it.
//
// A worker computes the request's cosmology scalars on the host, enqueues
// the pipeline (white noise generated on the device from the seed) and, when
// an output callback is set, copies the particles in chunks into two
// page-locked staging buffers, calling the callback for one chunk while the
// next is in flight.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/monofonic_gb300_batch.h"
#include "mf_request.h"
#include "mf_runtime.h"

using namespace mf;

namespace {

struct ShapeKey {
  int n, order, lattice, prec, pos64, id64;
  double L, z;
  bool operator==(const ShapeKey& o) const {
    return n == o.n && order == o.order && lattice == o.lattice && prec == o.prec && pos64 == o.pos64 &&
           id64 == o.id64 && L == o.L && z == o.z;
  }
};

ShapeKey key_of(const mf_ic_request& r) {
  return ShapeKey{r.ngrid, r.lpt_order, r.lattice, r.precision, r.pos64 ? 1 : 0, r.id64 ? 1 : 0, r.boxlen, r.zstart};
}

struct Pipe {
  mf_ctx* ctx = nullptr;
  mf_ic* ic = nullptr;
  ShapeKey key{};
  size_t bytes = 0;
  double last_used = 0;
  bool busy = false;
  cudaEvent_t g0 = nullptr, g1 = nullptr;
};

struct Req {
  mf_ic_request r{};
  mf_request_result res{};
  size_t need = 0;  // device footprint of a new pipeline for it
  bool done = false;
  bool cancel = false;  // set by mf_server_cancel while the request runs
};

struct Staging {
  void* buf[2] = {nullptr, nullptr};
  size_t bytes = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

void destroy_pipe(Pipe* p) {
  if (!p) return;
  if (p->ic) mf_ic_destroy(p->ic);
  if (p->g0) cudaEventDestroy(p->g0);
  if (p->g1) cudaEventDestroy(p->g1);
  if (p->ctx) mf_ctx_destroy(p->ctx);
  delete p;
}

}  // namespace

struct mf_server {
  int device = 0;
  mf_server_config cfg{};
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;
  std::vector<Req*> reqs;  // by id
  std::vector<Pipe*> pipes;  // every live pipeline (busy or pooled)
  std::vector<std::thread> workers;
  size_t budget = 0, in_use = 0, peak = 0;
  int64_t completed = 0, failed = 0, running = 0;
  bool stop = false;
  std::string err;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // admission under mu: picks a request and its pipeline (pooled, or a new
  // one whose bytes are reserved); idle pipelines to evict go to *evict
  bool admit(int64_t* id, Pipe** pipe, size_t* reserve, std::vector<Pipe*>* evict) {
    const double t = now();
    size_t qi = 0;
    for (auto it = queue.begin(); it != queue.end(); ++it, ++qi) {
      Req* q = reqs[*it];
      const bool head_starved = (qi == 0) && (t - q->res.t_submit > cfg.starvation_s);
      const ShapeKey k = key_of(q->r);
      Pipe* idle = nullptr;
      for (Pipe* p : pipes)
        if (!p->busy && p->key == k) { idle = p; break; }
      if (idle) {
        idle->busy = true;
        *id = *it;
        *pipe = idle;
        *reserve = 0;
        queue.erase(it);
        return true;
      }
      if (in_use + q->need > budget) {
        // evict idle pipelines, least recently used first, if that makes room
        size_t freeable = 0;
        for (Pipe* p : pipes)
          if (!p->busy) freeable += p->bytes;
        if (in_use - freeable + q->need <= budget) {
          while (in_use + q->need > budget) {
            Pipe* lru = nullptr;
            for (Pipe* p : pipes)
              if (!p->busy && (!lru || p->last_used < lru->last_used)) lru = p;
            for (size_t i = 0; i < pipes.size(); ++i)
              if (pipes[i] == lru) { pipes.erase(pipes.begin() + i); break; }
            in_use -= lru->bytes;
            evict->push_back(lru);
          }
        }
      }
      if (in_use + q->need <= budget) {
        in_use += q->need;
        if (in_use > peak) peak = in_use;
        *id = *it;
        *pipe = nullptr;
        *reserve = q->need;
        queue.erase(it);
        return true;
      }
      if (head_starved) return false;  // the head waits for room; nobody overtakes it
    }
    return false;
  }

  bool cancelled(const Req* q) {
    std::lock_guard<std::mutex> lk(mu);
    return q->cancel;
  }

  void finish(Req* q, int status) {
    std::lock_guard<std::mutex> lk(mu);
    q->res.status = status;
    q->res.t_done = now();
    q->done = true;
    --running;
    if (status == MF_OK) ++completed;
    else ++failed;
    cv_done.notify_all();
    cv_work.notify_all();
  }

  int run_request(Req* q, Pipe* p, Staging& st);
  void worker_loop();
};

int mf_server::run_request(Req* q, Pipe* p, Staging& st) {
  cudaSetDevice(device);
  mf_cosmo_scalars sc{};
  int rc = mf_cosmology_compute(&q->r.cosmo, q->r.zstart, &sc);
  if (rc != MF_OK) return rc;
  if ((rc = mf_ic_set_cosmology(p->ic, &sc)) != MF_OK) return rc;
  mf_ic_set_noise_seed(p->ic, q->r.seed);
  if (cancelled(q)) return MF_ERR_CANCELLED;
  cudaStream_t s = p->ctx->stream;
  cudaEventRecord(p->g0, s);
  if ((rc = mf_ic_enqueue(p->ic)) != MF_OK) return rc;
  cudaEventRecord(p->g1, s);
  if (cudaEventSynchronize(p->g1) != cudaSuccess) return MF_ERR_CUDA;
  if ((rc = mf_ctx_synchronize(p->ctx)) != MF_OK) return rc;  // bounded-wait error flag
  float ms = 0;
  cudaEventElapsedTime(&ms, p->g0, p->g1);
  mf_particles dev{};
  mf_ic_particles(p->ic, &dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    q->res.gpu_ms = ms;
    q->res.npart = dev.npart;
    q->res.t_gpu_done = now();
  }
  if (!cfg.output) return MF_OK;
  // stream the particles to the output callback in chunks
  const size_t rs = q->r.pos64 ? 8 : 4, is = q->r.id64 ? 8 : 4;
  const size_t per = 6 * rs + is;
  const int64_t chunk = cfg.chunk_particles;
  const size_t need = (size_t)chunk * per;
  if (st.bytes < need) {
    for (auto& b : st.buf)
      if (b) cudaFreeHost(b);
    st.buf[0] = st.buf[1] = nullptr;
    st.bytes = 0;
    for (auto& b : st.buf)
      if (cudaHostAlloc(&b, need, cudaHostAllocDefault) != cudaSuccess) return MF_ERR_OOM;
    st.bytes = need;
  }
  const int64_t np = dev.npart;
  const int64_t nch = (np + chunk - 1) / chunk;
  auto issue = [&](int64_t c) -> cudaError_t {
    const int64_t f = c * chunk, cnt = std::min<int64_t>(chunk, np - f);
    char* h = (char*)st.buf[c & 1];
    cudaError_t e = cudaMemcpyAsync(h, (char*)dev.pos + f * 3 * rs, cnt * 3 * rs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h + cnt * 3 * rs, (char*)dev.vel + f * 3 * rs, cnt * 3 * rs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h + cnt * 6 * rs, (char*)dev.ids + f * is, cnt * is, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(st.ev[c & 1], s);
    return e;
  };
  if (issue(0) != cudaSuccess) return MF_ERR_CUDA;
  for (int64_t c = 0; c < nch; ++c) {
    if (cancelled(q)) {  // let the copies in flight land before the buffers are reused
      cudaStreamSynchronize(s);
      return MF_ERR_CANCELLED;
    }
    if (c + 1 < nch && issue(c + 1) != cudaSuccess) return MF_ERR_CUDA;
    if (cudaEventSynchronize(st.ev[c & 1]) != cudaSuccess) return MF_ERR_CUDA;
    const int64_t f = c * chunk, cnt = std::min<int64_t>(chunk, np - f);
    char* h = (char*)st.buf[c & 1];
    mf_particles part{};
    part.pos = h;
    part.vel = h + cnt * 3 * rs;
    part.ids = h + cnt * 6 * rs;
    part.npart = cnt;
    part.location = MF_LOC_HOST;
    cfg.output(cfg.user, q->res.id, &part, f, cnt, c + 1 == nch ? 1 : 0);
    // the buffer of chunk c is reused by chunk c+2, issued after this call
  }
  return MF_OK;
}

void mf_server::worker_loop() {
  cudaSetDevice(device);
  Staging st;
  for (auto& e : st.ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  for (;;) {
    int64_t id = -1;
    Pipe* pipe = nullptr;
    size_t reserve = 0;
    std::vector<Pipe*> evict;
    {
      std::unique_lock<std::mutex> lk(mu);
      // re-check at least every 50 ms so that the starvation rule takes effect
      while (!stop && !admit(&id, &pipe, &reserve, &evict)) cv_work.wait_for(lk, std::chrono::milliseconds(50));
      if (stop && id < 0) break;
      ++running;
      reqs[id]->res.t_admit = now();
    }
    for (Pipe* p : evict) destroy_pipe(p);
    Req* q = reqs[id];
    int rc = MF_OK;
    if (!pipe) {  // a new pipeline in the reserved bytes
      pipe = new (std::nothrow) Pipe();
      if (!pipe) rc = MF_ERR_OOM;
      if (rc == MF_OK) rc = mf_ctx_create(device, &pipe->ctx);
      mf_cosmo_scalars sc{};
      if (rc == MF_OK) rc = mf_cosmology_compute(&q->r.cosmo, q->r.zstart, &sc);
      if (rc == MF_OK) {
        const mf_ic_params prm = request_params(q->r, sc);
        rc = mf_ic_create(pipe->ctx, &prm, &pipe->ic);
        if (rc != MF_OK) {
          std::lock_guard<std::mutex> lk(mu);
          err = std::string("request ") + std::to_string(id) + ": " + mf_last_error(pipe->ctx);
        }
      }
      if (rc == MF_OK && (cudaEventCreate(&pipe->g0) != cudaSuccess || cudaEventCreate(&pipe->g1) != cudaSuccess))
        rc = MF_ERR_CUDA;
      if (rc == MF_OK) {
        pipe->key = key_of(q->r);
        pipe->bytes = reserve;
        pipe->busy = true;
        std::lock_guard<std::mutex> lk(mu);
        pipes.push_back(pipe);
      } else {
        destroy_pipe(pipe);
        pipe = nullptr;
        std::lock_guard<std::mutex> lk(mu);
        in_use -= reserve;
      }
    }
    if (rc == MF_OK) rc = run_request(q, pipe, st);
    if (pipe) {
      std::lock_guard<std::mutex> lk(mu);
      pipe->busy = false;
      pipe->last_used = now();
      if (rc != MF_OK && err.empty()) err = std::string("request ") + std::to_string(id) + " failed: " + mf_last_error(pipe->ctx);
    }
    finish(q, rc);
  }
  for (auto& b : st.buf)
    if (b) cudaFreeHost(b);
  for (auto& e : st.ev)
    if (e) cudaEventDestroy(e);
}

extern "C" int mf_server_create(int device, const mf_server_config* cfg, mf_server** out) {
  if (!out) return MF_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return MF_ERR_CUDA;
  mf_server* s = new (std::nothrow) mf_server();
  if (!s) return MF_ERR_OOM;
  s->device = device;
  if (cfg) s->cfg = *cfg;
  if (s->cfg.nworkers <= 0) s->cfg.nworkers = 4;
  if (s->cfg.chunk_particles <= 0) s->cfg.chunk_particles = (int64_t)2 << 20;
  if (s->cfg.starvation_s <= 0) s->cfg.starvation_s = 2.0;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    delete s;
    return MF_ERR_CUDA;
  }
  s->budget = s->cfg.hbm_budget ? s->cfg.hbm_budget : (size_t)(0.9 * (double)fr);
  s->t0 = std::chrono::steady_clock::now();
  for (int w = 0; w < s->cfg.nworkers; ++w) s->workers.emplace_back([s] { s->worker_loop(); });
  *out = s;
  return MF_OK;
}

extern "C" int mf_server_submit(mf_server* s, const mf_ic_request* r, int64_t* id) {
  if (!s || !r) return MF_ERR_ARG;
  int rc = check_request(*r);
  if (rc != MF_OK) return rc;
  // footprint with placeholder scalars (the sizes do not depend on them)
  mf_cosmo_scalars sc{};
  sc.pnorm = 1;
  sc.Dplus = 1;
  const mf_ic_params p = request_params(*r, sc);
  size_t need = 0;
  if ((rc = mf_ic_device_footprint(&p, &need)) != MF_OK) return rc;
  Req* q = new (std::nothrow) Req();
  if (!q) return MF_ERR_OOM;
  q->r = *r;
  q->need = need;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) {
    delete q;
    return MF_ERR_STATE;
  }
  if (need > s->budget) {
    delete q;
    s->err = "mf_server_submit: the request needs more device memory than the budget";
    return MF_ERR_OOM;
  }
  q->res.id = (int64_t)s->reqs.size();
  q->res.t_submit = s->now();
  s->reqs.push_back(q);
  s->queue.push_back(q->res.id);
  if (id) *id = q->res.id;
  s->cv_work.notify_one();
  return MF_OK;
}

extern "C" int mf_server_wait(mf_server* s, int64_t id, mf_request_result* out, double timeout_s) {
  if (!s) return MF_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->reqs.size()) return MF_ERR_ARG;
  // looked up again after every wake-up: another thread may release the record
  auto pred = [&] { return !s->reqs[id] || s->reqs[id]->done; };
  if (timeout_s < 0) s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return MF_ERR_TIMEOUT;
  const Req* q = s->reqs[id];
  if (!q) return MF_ERR_STATE;
  if (out) *out = q->res;
  return MF_OK;
}

extern "C" int mf_server_release(mf_server* s, int64_t id) {
  if (!s) return MF_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->reqs.size()) return MF_ERR_ARG;
  Req* q = s->reqs[id];
  if (!q || !q->done) return MF_ERR_STATE;
  delete q;
  s->reqs[id] = nullptr;
  s->cv_done.notify_all();  // waiters on this id return MF_ERR_STATE
  return MF_OK;
}

extern "C" int mf_server_poll(mf_server* s, int64_t id, mf_request_result* out, int* done) {
  if (!s || !done) return MF_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->reqs.size()) return MF_ERR_ARG;
  const Req* q = s->reqs[id];
  if (!q) return MF_ERR_STATE;
  *done = q->done ? 1 : 0;
  if (q->done && out) *out = q->res;
  return MF_OK;
}

extern "C" int mf_server_cancel(mf_server* s, int64_t id) {
  if (!s) return MF_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (int64_t)s->reqs.size()) return MF_ERR_ARG;
  Req* q = s->reqs[id];
  if (!q || q->done) return MF_ERR_STATE;
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
    if (*it == id) {  // never admitted: finishes now
      s->queue.erase(it);
      q->res.status = MF_ERR_CANCELLED;
      q->res.t_done = s->now();
      q->done = true;
      ++s->failed;
      s->cv_done.notify_all();
      s->cv_work.notify_all();
      return MF_OK;
    }
  q->cancel = true;  // running: stops at its next stage boundary
  return MF_OK;
}

extern "C" int mf_server_drain(mf_server* s, double timeout_s) {
  if (!s) return MF_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto pred = [&] { return s->completed + s->failed == (int64_t)s->reqs.size(); };
  if (timeout_s < 0) s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return MF_ERR_TIMEOUT;
  return MF_OK;
}

extern "C" int mf_server_stats_get(mf_server* s, mf_server_stats* o) {
  if (!s || !o) return MF_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  o->submitted = (int64_t)s->reqs.size();
  o->completed = s->completed;
  o->failed = s->failed;
  o->queued = (int64_t)s->queue.size();
  o->running = s->running;
  o->bytes_in_use = s->in_use;
  o->bytes_budget = s->budget;
  o->peak_bytes = s->peak;
  o->pooled_pipelines = (int)s->pipes.size();
  o->t_now = s->now();
  return MF_OK;
}

extern "C" double mf_server_now(const mf_server* s) { return s ? s->now() : 0.0; }

extern "C" const char* mf_server_last_error(const mf_server* s) { return s ? s->err.c_str() : "null server"; }

extern "C" int mf_server_destroy(mf_server* s) {
  if (!s) return MF_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    // requests that were never admitted are cancelled
    for (int64_t id : s->queue) {
      Req* q = s->reqs[id];
      q->res.status = MF_ERR_CANCELLED;
      q->res.t_done = s->now();
      q->done = true;
      ++s->failed;
    }
    s->queue.clear();
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  for (auto& t : s->workers) t.join();
  cudaSetDevice(s->device);
  for (Pipe* p : s->pipes) destroy_pipe(p);
  for (Req* q : s->reqs) delete q;
  delete s;
  return MF_OK;
}
