"""Several GPUs of one node: replicas only.

A single IC does not shard without the global transposes of the reference's
slab decomposition (src/grid_fft.cc:115-189), and batches and serving streams
are independent realizations, so every rank runs whole realizations on its own
GPU.  Ranks meet only at a barrier and at reductions of their timings; no
collective touches the data path.  The launcher's environment (RANK,
WORLD_SIZE, LOCAL_RANK, MASTER_ADDR, MASTER_PORT) selects the rank; NCCL is the
GPU backend, gloo serves host-only use (tests).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Any


@dataclass
class Replicas:
    world: int
    rank: int
    local: int
    backend: str | None
    dist: Any = None

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x: float, op) -> float:
        if self.dist is None:
            return float(x)
        import torch
        dev = torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max_over_ranks(self, x: float) -> float:
        """the slowest rank's value (timings: max over ranks)"""
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.MAX)

    def sum_over_ranks(self, x: float) -> float:
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.SUM)

    def aggregate_rate(self, units_per_rank: float, seconds: float) -> float:
        """whole-job throughput: the units all ranks processed over the
        slowest rank's time"""
        total = self.sum_over_ranks(units_per_rank)
        slowest = self.max_over_ranks(seconds)
        return total / slowest

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def init(backend: str = "nccl") -> Replicas:
    """join the job described by the launcher's environment; a single process
    (WORLD_SIZE unset or 1) needs no process group"""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    r = Replicas(world, rank, local, backend if world > 1 else None)
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
        r.dist = dist
    return r


# ---------------------------------------------------------------------------
# replica serving over a shared queue
# ---------------------------------------------------------------------------
class ClaimQueue:
    """One request queue shared by the ranks of a job (one process per GPU):
    a torch.distributed Store holds the requests in arrival order and a few
    counters; any process may append (push), and every worker takes the next
    unclaimed request with one atomic add on the head counter (claim), so a
    request is served exactly once and faster replicas simply take more.
    Requests and results are strings (e.g. JSON)."""

    def __init__(self, store, prefix: str = "mfq"):
        self.store, self.p = store, prefix

    def push(self, payload: str) -> int:
        """append a request; returns its index (arrival order)"""
        idx = self.store.add(f"{self.p}/reserve", 1) - 1
        self.store.set(f"{self.p}/req/{idx}", payload)
        # the ready flag is written after the payload, so a claimer never reads a half-written slot
        self.store.add(f"{self.p}/ready/{idx}", 1)
        return idx

    def close_input(self):
        """no more requests will be pushed"""
        self.store.set(f"{self.p}/closed", "1")

    def claim(self, timeout_s: float = 60.0, poll_s: float = 0.001):
        """(index, payload) of the next unclaimed request, or None once the
        input is closed and every pushed request has been claimed"""
        import time
        idx = self.store.add(f"{self.p}/head", 1) - 1
        t0 = time.monotonic()
        while True:
            if self.store.check([f"{self.p}/ready/{idx}"]):
                return idx, self.store.get(f"{self.p}/req/{idx}").decode()
            if self.store.check([f"{self.p}/closed"]) and idx >= self.store.add(f"{self.p}/reserve", 0):
                return None
            if time.monotonic() - t0 > timeout_s:
                raise TimeoutError(f"ClaimQueue: request {idx} did not arrive within {timeout_s} s")
            time.sleep(poll_s)

    def complete(self, idx: int, result: str):
        self.store.set(f"{self.p}/done/{idx}", result)
        self.store.add(f"{self.p}/ndone", 1)

    def result(self, idx: int):
        k = f"{self.p}/done/{idx}"
        return self.store.get(k).decode() if self.store.check([k]) else None

    def completed(self) -> int:
        return self.store.add(f"{self.p}/ndone", 0)


class ReplicaServer:
    """Replica serving inside one process: one device server per GPU, all fed
    from one FIFO queue.  Each device has a dispatcher thread that takes the
    queue's head whenever fewer than `depth` of its requests are in flight
    (its server's own footprint admission then overlaps them on the device),
    so a less loaded or faster device takes more work; a collector thread per
    device moves finished requests to the results.  `make_server(device)`
    returns an object with the Server interface (submit / poll / close)."""

    def __init__(self, devices, make_server, depth: int = 4, poll_s: float = 0.0005):
        import collections
        import threading
        self.devices = list(devices)
        self.servers = [make_server(d) for d in self.devices]
        self.depth, self.poll_s = depth, poll_s
        self.queue = collections.deque()
        self.cv = threading.Condition()
        self.inflight = [dict() for _ in self.devices]  # per device: {server request id: global id}
        self.results, self.placement, self.order = {}, {}, []
        self.next_id = 0
        self.running = True
        self.threads = []
        for i in range(len(self.devices)):
            for fn in (self._dispatch, self._collect):
                t = threading.Thread(target=fn, args=(i,), daemon=True)
                t.start()
                self.threads.append(t)

    def submit(self, req) -> int:
        with self.cv:
            gid = self.next_id
            self.next_id += 1
            self.queue.append((gid, req))
            self.cv.notify_all()
        return gid

    def _dispatch(self, i):
        srv = self.servers[i]
        while True:
            with self.cv:
                while self.running and (not self.queue or len(self.inflight[i]) >= self.depth):
                    self.cv.wait(0.05)
                if not self.running:
                    return
                gid, req = self.queue.popleft()
                self.order.append(gid)
                rid = srv.submit(req)
                self.inflight[i][rid] = gid
                self.placement[gid] = i

    def _collect(self, i):
        import time
        srv = self.servers[i]
        while True:
            with self.cv:
                if not self.running:
                    return
                pending = list(self.inflight[i].items())
            done = []
            for rid, gid in pending:
                r = srv.poll(rid)
                if r is not None:
                    done.append((rid, gid, r))
            if done:
                with self.cv:
                    for rid, gid, r in done:
                        del self.inflight[i][rid]
                        self.results[gid] = dict(r, device=self.devices[i])
                    self.cv.notify_all()
            else:
                time.sleep(self.poll_s)

    def wait(self, gid: int, timeout_s: float = 60.0) -> dict:
        import time
        t0 = time.monotonic()
        with self.cv:
            while gid not in self.results:
                left = timeout_s - (time.monotonic() - t0)
                if left <= 0:
                    raise TimeoutError(f"request {gid} not finished within {timeout_s} s")
                self.cv.wait(min(left, 0.05))
            return self.results[gid]

    def drain(self, timeout_s: float = 600.0):
        import time
        t0 = time.monotonic()
        with self.cv:
            while self.queue or any(self.inflight):
                if time.monotonic() - t0 > timeout_s:
                    raise TimeoutError("ReplicaServer.drain")
                self.cv.wait(0.05)

    def per_device(self) -> dict:
        out = {d: 0 for d in self.devices}
        for gid, i in self.placement.items():
            out[self.devices[i]] += 1
        return out

    def close(self):
        with self.cv:
            self.running = False
            self.cv.notify_all()
        for t in self.threads:
            t.join(timeout=5)
        for s in self.servers:
            s.close()
