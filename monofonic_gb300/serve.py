"""Many realizations on one GPU (include/monofonic_gb300_batch.h): a recorded
batch (one CUDA graph launch over all realizations) and a continuous-batching
IC server with admission by device-memory footprint.

Each request carries the keys of one ic_generator::run (src/ic_generator.cc:90):
[setup] GridRes/BoxLength/zstart/LPTorder/ParticleLoad, [cosmology], [random]
seed; the white noise is the project RNG plugin (mf_white_noise_host), made on
the device from the seed.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import lib, MFError
from .ic import Cosmology, LATTICES


@dataclass
class Request:
    ngrid: int
    boxlen: float
    zstart: float = 24.0
    lpt_order: int = 3
    lattice: str = "sc"
    precision: str = "f32"
    cosmology: Cosmology = field(default_factory=Cosmology)
    seed: int = 12345
    pos64: bool = True
    id64: bool = True

    def to_c(self):
        r = L.mf_ic_request()
        r.ngrid = self.ngrid
        r.boxlen = self.boxlen
        r.zstart = self.zstart
        r.lpt_order = self.lpt_order
        r.lattice = LATTICES[self.lattice]
        r.precision = L.MF_PREC_F64 if self.precision == "f64" else L.MF_PREC_F32
        r.cosmo = self.cosmology.to_c()
        r.seed = int(self.seed)
        r.pos64 = int(self.pos64)
        r.id64 = int(self.id64)
        return r

    @property
    def npart(self) -> int:
        return self.ngrid ** 3 * (1 << LATTICES[self.lattice])


def _particles_to_host(p: "L.mf_particles", req: Request):
    rt = np.float64 if req.pos64 else np.float32
    it = np.uint64 if req.id64 else np.uint32
    n = int(p.npart)
    pos = np.empty((n, 3), dtype=rt)
    vel = np.empty((n, 3), dtype=rt)
    ids = np.empty(n, dtype=it)
    for a, src in ((pos, p.pos), (vel, p.vel), (ids, p.ids)):
        rc = lib().mf_copy_to_host(a.ctypes.data, src, a.nbytes)
        if rc != L.MF_OK:
            raise MFError(rc, "mf_copy_to_host")
    return pos, vel, ids


class Batch:
    """All realizations recorded into one CUDA graph over nstreams streams."""

    def __init__(self, requests, nstreams: int = 8, device: int = 0, autotune: bool = False):
        self.requests = list(requests)
        arr = (L.mf_ic_request * len(self.requests))(*[r.to_c() for r in self.requests])
        p = C.c_void_p()
        rc = lib().mf_batch_create(int(device), arr, len(self.requests), int(nstreams), 1 if autotune else 0,
                                   C.byref(p))
        if rc != L.MF_OK:
            msg = lib().mf_batch_last_error(None)
            raise MFError(rc, msg.decode() if msg else "mf_batch_create")
        self.ptr = p

    def _check(self, rc, what):
        if rc != L.MF_OK:
            msg = lib().mf_batch_last_error(self.ptr)
            raise MFError(rc, f"{what}: {msg.decode() if msg else ''}")

    def run(self) -> float:
        """one graph launch over every realization; returns device ms"""
        ms = C.c_double()
        self._check(lib().mf_batch_run(self.ptr, C.byref(ms)), "mf_batch_run")
        return ms.value

    def set_items(self, first: int, cosmologies=None, seeds=None, nthreads: int = 0):
        count = len(cosmologies) if cosmologies is not None else len(seeds)
        cz = (L.mf_cosmo_params * count)(*[c.to_c() for c in cosmologies]) if cosmologies is not None else None
        sd = (C.c_uint64 * count)(*[int(s) for s in seeds]) if seeds is not None else None
        self._check(lib().mf_batch_set_items(self.ptr, int(first), count, cz, sd, int(nthreads)), "mf_batch_set_items")
        for i in range(count):
            r = self.requests[first + i]
            if cosmologies is not None:
                r.cosmology = cosmologies[i]
            if seeds is not None:
                r.seed = int(seeds[i])

    def particles(self, i: int):
        """(pos, vel, ids) of realization i on the host"""
        p = L.mf_particles()
        self._check(lib().mf_batch_particles(self.ptr, int(i), C.byref(p)), "mf_batch_particles")
        return _particles_to_host(p, self.requests[i])

    @property
    def tuning(self) -> str:
        """the autotuner's report (one line per pass kind and shape)"""
        r = lib().mf_batch_tuning(self.ptr)
        return r.decode() if r else ""

    def info(self):
        nodes, kern, nb = C.c_int(), C.c_longlong(), C.c_size_t()
        self._check(lib().mf_batch_info(self.ptr, C.byref(nodes), C.byref(kern), C.byref(nb)), "mf_batch_info")
        return {"graph_nodes": nodes.value, "kernels": kern.value, "device_bytes": nb.value}

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching IC server.

    output: "collect" keeps every request's particles as numpy arrays
    (self.results[id] = (pos, vel, ids)); "count" reads the particles back in
    chunks and only counts them; None leaves them on the device."""

    def __init__(self, nworkers: int = 4, hbm_budget: int = 0, chunk_particles: int = 0, output: str | None = "count",
                 starvation_s: float = 0.0, device: int = 0):
        self.output = output
        self.results = {}
        self.bytes_out = 0
        self._lock = threading.Lock()
        self._reqs = {}
        cfg = L.mf_server_config()
        cfg.nworkers = int(nworkers)
        cfg.hbm_budget = int(hbm_budget)
        cfg.chunk_particles = int(chunk_particles)
        cfg.starvation_s = float(starvation_s)
        self._cb = L.MF_OUTPUT_FN(self._on_chunk) if output else L.MF_OUTPUT_FN()
        cfg.output = self._cb
        cfg.user = None
        p = C.c_void_p()
        rc = lib().mf_server_create(int(device), C.byref(cfg), C.byref(p))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_create")
        self.ptr = p

    def _on_chunk(self, user, rid, part, first, count, last):
        p = part.contents
        with self._lock:  # submit() holds the lock until the request is registered
            req = self._reqs[rid]
            rs = 8 if req.pos64 else 4
            is_ = 8 if req.id64 else 4
            self.bytes_out += count * (6 * rs + is_)
            arrays = self.results.get(rid)
        if self.output != "collect":
            return
        pos, vel, ids = arrays
        C.memmove(pos.ctypes.data + first * 3 * rs, p.pos, count * 3 * rs)
        C.memmove(vel.ctypes.data + first * 3 * rs, p.vel, count * 3 * rs)
        C.memmove(ids.ctypes.data + first * is_, p.ids, count * is_)

    def submit(self, req: Request) -> int:
        rid = C.c_int64()
        # the output arrays must exist before the first chunk can arrive
        with self._lock:
            rc = lib().mf_server_submit(self.ptr, C.byref(req.to_c()), C.byref(rid))
            if rc != L.MF_OK:
                msg = lib().mf_server_last_error(self.ptr)
                raise MFError(rc, msg.decode() if msg else "mf_server_submit")
            self._reqs[rid.value] = req
            if self.output == "collect":
                rt = np.float64 if req.pos64 else np.float32
                it = np.uint64 if req.id64 else np.uint32
                n = req.npart
                self.results[rid.value] = (np.empty((n, 3), rt), np.empty((n, 3), rt), np.empty(n, it))
        return rid.value

    def wait(self, rid: int, timeout_s: float = -1.0) -> dict:
        r = L.mf_request_result()
        rc = lib().mf_server_wait(self.ptr, int(rid), C.byref(r), float(timeout_s))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_wait")
        return {f: getattr(r, f) for f, _ in r._fields_}

    def poll(self, rid: int) -> dict | None:
        """the request's result if it has finished, else None (never blocks)"""
        r = L.mf_request_result()
        done = C.c_int()
        rc = lib().mf_server_poll(self.ptr, int(rid), C.byref(r), C.byref(done))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_poll")
        return {f: getattr(r, f) for f, _ in r._fields_} if done.value else None

    def cancel(self, rid: int):
        """cancel a queued request (it never runs) or stop a running one at its
        next stage boundary; MFError(MF_ERR_STATE) once it has finished"""
        rc = lib().mf_server_cancel(self.ptr, int(rid))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_cancel")

    def release(self, rid: int):
        """free a finished request's record here and in the server (its
        collected particles are dropped); its id is then unknown"""
        rc = lib().mf_server_release(self.ptr, int(rid))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_release")
        with self._lock:
            self._reqs.pop(rid, None)
            self.results.pop(rid, None)

    def drain(self, timeout_s: float = -1.0):
        rc = lib().mf_server_drain(self.ptr, float(timeout_s))
        if rc != L.MF_OK:
            raise MFError(rc, "mf_server_drain")

    def stats(self) -> dict:
        st = L.mf_server_stats()
        lib().mf_server_stats_get(self.ptr, C.byref(st))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def now(self) -> float:
        return lib().mf_server_now(self.ptr)

    def last_error(self) -> str:
        m = lib().mf_server_last_error(self.ptr)
        return m.decode() if m else ""

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
