/*
 * monofonic_gb300_batch.h -- many realizations on one GPU: a recorded batch
 * (one CUDA graph over all realizations) and a continuous-batching IC server.
 *
 * The reference has no batch or server interface: ic_generator::run
 * (src/ic_generator.cc:90) makes one realization per process from a config
 * file.  Each request here carries the [setup]/[cosmology]/[random] keys of
 * one such run; the pipeline is the one of monofonic_gb300_ic.h and the
 * particles go to an output callback in the role of
 * output_plugin::write_particle_data (include/output_plugin.hh:59-62).
 */
#ifndef MONOFONIC_GB300_BATCH_H
#define MONOFONIC_GB300_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "monofonic_gb300_ic.h"

#ifdef __cplusplus
extern "C" {
#endif

/* one realization: [setup] GridRes, BoxLength, zstart, LPTorder,
 * ParticleLoad; [cosmology]; [random] seed; precision of the pipeline */
typedef struct {
  int ngrid;
  double boxlen;
  double zstart;
  int lpt_order;
  int lattice;        /* MF_LATTICE_* */
  int precision;      /* MF_PREC_F32 (bulk) or MF_PREC_F64 (plain) */
  mf_cosmo_params cosmo;
  uint64_t seed;      /* white noise of mf_white_noise_host, made on the device */
  int pos64, id64;    /* output_plugin::has_64bit_reals / has_64bit_ids */
} mf_ic_request;

/* ---- recorded batch -------------------------------------------------------
 * Every realization gets its own device pipeline; the realizations are
 * spread over nstreams streams (largest first onto the least loaded stream)
 * and the whole batch is recorded into one CUDA graph, so that a run is one
 * graph launch.  New seeds and cosmologies replay the same graph. */
typedef struct mf_batch mf_batch;

enum { MF_BATCH_AUTOTUNE = 1 };
/* flags: MF_BATCH_AUTOTUNE runs mf_autotune for every distinct grid size and
 * precision of the batch before the graph is recorded */
int mf_batch_create(int device, const mf_ic_request* items, int nitems, int nstreams, int flags, mf_batch** out);
int mf_batch_destroy(mf_batch* b);
/* new cosmology and seed of realizations [first, first+count) for the next
 * run (grid, box, order, lattice and precision stay); cosmology scalars are
 * computed on nthreads host threads (<= 0: all) */
int mf_batch_set_items(mf_batch* b, int first, int count, const mf_cosmo_params* cosmo, const uint64_t* seeds,
                       int nthreads);
/* one launch of the recorded graph; waits for it; *ms = device time */
int mf_batch_run(mf_batch* b, double* ms);
/* device buffers of realization i after a run */
int mf_batch_particles(mf_batch* b, int i, mf_particles* out);
/* graph nodes, kernel launches per run, device bytes of all pipelines */
int mf_batch_info(mf_batch* b, int* graph_nodes, long long* kernels, size_t* device_bytes);
/* the autotuner's report (empty without MF_BATCH_AUTOTUNE) */
const char* mf_batch_tuning(const mf_batch* b);
/* message of the last failure on b; with b == NULL, of the last failed
 * mf_batch_create on the calling thread */
const char* mf_batch_last_error(const mf_batch* b);

/* ---- continuous-batching server --------------------------------------------
 * nworkers host threads, each with its own stream; a request is admitted when
 * a worker is free and its pipeline fits the device-memory budget (the
 * mf_ic_device_footprint of the pipeline: fields, the 3/2-padded convolution
 * buffers and the particles), reusing an idle pipeline of the same shape when
 * one is pooled.  Requests admitted while others run overlap on the device.
 * The particles of a finished request are copied to page-locked host memory
 * in chunks and handed to the output callback in order. */
typedef struct mf_server mf_server;

/* one chunk of a request's particles (host memory valid during the call):
 * particles [first, first+count) of npart; last != 0 on the final chunk */
typedef void (*mf_output_fn)(void* user, int64_t request_id, const mf_particles* chunk, int64_t first,
                             int64_t count, int last);

typedef struct {
  int nworkers;            /* streams / concurrently running requests (>= 1) */
  size_t hbm_budget;       /* bytes of device memory for pipelines; 0: 90% of free */
  int64_t chunk_particles; /* particles per output chunk; 0: 8 Mi */
  mf_output_fn output;     /* NULL: particles stay on the device (not read back) */
  void* user;
  double starvation_s;     /* a request waiting longer than this blocks
                              admission of later ones until it fits; 0: 2 s */
} mf_server_config;

typedef struct {
  int64_t id;
  int status;              /* MF_OK or the failing status */
  int64_t npart;
  double t_submit, t_admit, t_gpu_done, t_done;  /* seconds on the server's clock */
  double gpu_ms;           /* device time of the pipeline (CUDA events) */
} mf_request_result;

typedef struct {
  int64_t submitted, completed, failed, queued, running;
  size_t bytes_in_use, bytes_budget, peak_bytes;
  int pooled_pipelines;
  double t_now;
} mf_server_stats;

int mf_server_create(int device, const mf_server_config* cfg, mf_server** out);
/* enqueue a request; returns its id in *id (ids start at 0) */
int mf_server_submit(mf_server* s, const mf_ic_request* req, int64_t* id);
/* wait until request id has finished (timeout_s < 0: no limit);
 * MF_ERR_TIMEOUT if it has not finished in time, MF_ERR_STATE once released */
int mf_server_wait(mf_server* s, int64_t id, mf_request_result* out, double timeout_s);
/* free the record of a finished request (a long-running server otherwise
 * keeps one per request until mf_server_destroy); its id then answers
 * MF_ERR_STATE.  MF_ERR_STATE if it has not finished or was released */
int mf_server_release(mf_server* s, int64_t id);
/* non-blocking status of request id: *done = 1 and *out filled (out may be
 * NULL) once it has finished, else *done = 0; MF_ERR_STATE once released */
int mf_server_poll(mf_server* s, int64_t id, mf_request_result* out, int* done);
/* cancel request id.  A queued request is taken out of the queue and finishes
 * at once with MF_ERR_CANCELLED.  A running request finishes with
 * MF_ERR_CANCELLED at its next stage boundary (before its pipeline is
 * enqueued, or between two output chunks); device work already enqueued
 * completes.  MF_ERR_STATE if the request has already finished. */
int mf_server_cancel(mf_server* s, int64_t id);
/* wait until every submitted request has finished */
int mf_server_drain(mf_server* s, double timeout_s);
int mf_server_stats_get(mf_server* s, mf_server_stats* out);
/* seconds on the server's clock (the t_* fields of mf_request_result) */
double mf_server_now(const mf_server* s);
const char* mf_server_last_error(const mf_server* s);
int mf_server_destroy(mf_server* s);

#ifdef __cplusplus
}
#endif
#endif /* MONOFONIC_GB300_BATCH_H */
