"""Several GPUs of one node run replicas (monofonic_gb300/replicas.py): ranks
meet only at a barrier and at reductions of their timings.  Two gloo ranks on
the CPU exercise that host logic; the reference arm of bench.py prints on rank
0 only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from monofonic_gb300 import replicas
    job = replicas.init("gloo")
    assert job.world == world and job.rank == rank and job.dist is not None
    mx = job.max_over_ranks(1.5 + rank)
    sm = job.sum_over_ranks(10.0 * (rank + 1))
    # 100 units per rank, the slowest rank took 3 s: 200 / 3 units per second
    rate = job.aggregate_rate(100.0, 2.0 + rank)
    job.barrier()
    job.close()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{mx} {sm} {rate}")


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        mx, sm, rate = map(float, (tmp_path / f"rank{r}.txt").read_text().split())
        assert mx == 2.5 and sm == 30.0
        assert rate == pytest.approx(200.0 / 3.0, rel=1e-15)


def test_single_process_needs_no_group(monkeypatch):
    from monofonic_gb300 import replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    job = replicas.init("gloo")
    assert job.world == 1 and job.dist is None and job.backend is None
    assert job.max_over_ranks(4.0) == 4.0 and job.aggregate_rate(10.0, 2.0) == 5.0
    job.barrier()
    job.close()


def test_reference_arm_prints_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_bench_gpus_2_starts_two_ranks():
    """bench.py --gpus 2 outside a launcher starts two ranks itself (the stub
    arm runs the GPU arm's rank bookkeeping on gloo) and reports the real
    world size"""
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE")}
    p = subprocess.run([sys.executable, "bench.py", "--impl", "stub", "--gpus", "2", "--steps", "3", "--warmup", "0"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["ranks_joined"] == 2
    # both ranks' units over the slowest rank's time
    assert d["value"] == pytest.approx(2 * 3000.0 / (d["ms_per_step"] * 3 / 1e3), rel=1e-9)


# ---------------------------------------------------------------------------
# replica serving over one shared queue (monofonic_gb300/replicas.py)
# ---------------------------------------------------------------------------
class _FakeServer:
    """a device server without a device: each request takes cost / speed
    seconds on a worker thread (the Server interface: submit / poll / close)"""

    def __init__(self, device, speed):
        import threading
        self.device, self.speed = device, speed
        self.done, self.next, self.lock = {}, 0, threading.Lock()
        self.sem = threading.Semaphore(2)  # two requests overlap on a fake device

    def submit(self, req):
        import threading
        import time
        with self.lock:
            rid = self.next
            self.next += 1

        def work():
            with self.sem:
                time.sleep(req["cost"] / self.speed)
            with self.lock:
                self.done[rid] = {"status": 0, "key": req["key"]}
        threading.Thread(target=work, daemon=True).start()
        return rid

    def poll(self, rid):
        with self.lock:
            return self.done.get(rid)

    def close(self):
        pass


def test_replica_server_shares_one_queue():
    """two fake devices (one four times faster) pull from one FIFO queue:
    every request finishes exactly once with its own result, requests leave
    the queue in arrival order, and the faster device serves more of them"""
    from monofonic_gb300.replicas import ReplicaServer
    speeds = {0: 1.0, 1: 4.0}
    rs = ReplicaServer([0, 1], lambda d: _FakeServer(d, speeds[d]), depth=2)
    gids = [rs.submit({"cost": 0.01, "key": k}) for k in range(60)]
    rs.drain(60.0)
    res = [rs.wait(g, 10.0) for g in gids]
    assert [r["key"] for r in res] == list(range(60))
    assert rs.order == sorted(rs.order) and len(rs.order) == 60
    per = rs.per_device()
    assert sum(per.values()) == 60 and per[1] > per[0]
    rs.close()


def _claim_rank(rank, world, port, out_dir, nreq):
    import json
    import threading
    import time
    import torch.distributed as dist
    from monofonic_gb300.replicas import ClaimQueue
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo")
    store = dist.distributed_c10d._get_default_store()
    q = ClaimQueue(store, prefix="t")
    if rank == 0:  # the submitter: requests arrive while the replicas work
        def feed():
            for i in range(nreq):
                q.push(json.dumps({"key": i}))
                time.sleep(0.001)
            q.close_input()
        th = threading.Thread(target=feed)
        th.start()
    mine = []
    per_req = 0.002 if rank == 0 else 0.008  # rank 1 is four times slower
    while True:
        c = q.claim(timeout_s=30.0)
        if c is None:
            break
        idx, payload = c
        time.sleep(per_req)
        q.complete(idx, json.dumps({"key": json.loads(payload)["key"], "rank": rank}))
        mine.append(idx)
    if rank == 0:
        th.join()
    dist.barrier()
    if rank == 0:
        results = [json.loads(q.result(i)) for i in range(nreq)]
        assert [r["key"] for r in results] == list(range(nreq)) and q.completed() == nreq
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"claims{rank}.json"), "w") as f:
        json.dump(mine, f)


def test_claim_queue_two_gloo_ranks(tmp_path):
    """two ranks serve one queue that a third party keeps filling: every
    request is claimed by exactly one rank, and the faster rank takes more"""
    import json
    import torch.multiprocessing as mp
    nreq = 80
    mp.spawn(_claim_rank, args=(2, _free_port(), str(tmp_path), nreq), nprocs=2, join=True)
    c0 = json.loads((tmp_path / "claims0.json").read_text())
    c1 = json.loads((tmp_path / "claims1.json").read_text())
    assert sorted(c0 + c1) == list(range(nreq))
    assert len(c0) > len(c1) > 0
