#!/usr/bin/env python3
"""Benchmark: 3LPT particles/s at 512^3 on one GB300, FP32-bulk vs FP64 plain.

Workload (one "step" = one full initial-condition pass over one synthetic
realization): 3LPT, Orszag 3/2 dealiasing (padded 768^3 convolutions), BCC
lattice of 2 x 512^3 particles, box 1000 Mpc/h, z_start = 24, Eisenstein & Hu
transfer function, seeded N(0,1) white noise (synthetic; no dataset).

  value   particles/s of the FP32-bulk form, white noise already resident in
          HBM when the timed region starts, particles (positions, velocities,
          IDs) resident in HBM when it ends; CUDA events on the pipeline's
          stream; the working set (>16 GB) is far larger than L2.
  e2e     the same through the public C ABI (mf_ic_set_noise +
          mf_ic_run_async, mf_ic_wait after the last step) with the noise
          copied from page-locked host memory and all particles copied back
          to page-locked host memory every step; a run's particle copies
          overlap the next run's fields (sync_ms_per_step: one synchronous
          mf_ic_run per step instead).
  fp64    the plain FP64 form on the same workload (positions in double).

--impl reference times the reference's CPU path on the host cores: whole
initial conditions of the oracle port (numpy/scipy FP64, all host threads;
pinned to the reference's own program by the CPU tests) at N = 128 with the
workload's box per cell, one whole IC per step, nothing extrapolated.

Multi-GPU: every rank runs an independent realization (replicas; no
collectives on the data path); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3LPT particles/s at 512^3: FP32-bulk vs FP64 plain (1 GB300); p50/p99 IC latency"
UNIT = "particles/s"

WORKLOAD = dict(ngrid=512, boxlen=1000.0, zstart=24.0, lpt_order=3, lattice="bcc", plt=True)
COSMO = dict(Omega_m=0.3099, Omega_b=0.0488, h=0.6774, sigma_8=0.8102, n_s=0.9667)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    # "stub": the rank bookkeeping alone on gloo/CPU (no GPU work), for testing
    # that --gpus N starts N ranks
    ap.add_argument("--impl", default="mf", choices=["mf", "reference", "stub"])
    ap.add_argument("--ngrid", type=int, default=512)
    ap.add_argument("--ref-ngrid", type=int, default=128, help="grid of one reference-arm step (a whole IC)")
    ap.add_argument("--ref-plt-ngrid", type=int, default=64, help="PLT table mesh of the reference arm")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-output", action="store_true")
    ap.add_argument("--batch-items", type=int, default=96)
    ap.add_argument("--batch-streams", type=int, default=8)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-seconds-fp64", type=float, default=60.0)
    ap.add_argument("--detail", default=None, help="file for the full per-kernel / batch / serving detail")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-workers", type=int, default=4)
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic bytes per launch of each kernel kind for one 3LPT IC
# ---------------------------------------------------------------------------
def algorithmic_bytes_ic(n: int, prec_bytes: int, overload: int = 2, plt: bool = True) -> dict:
    """Unique bytes each kernel kind must read and write for one 3LPT IC of the
    shared-source pipeline (each element once; re-reads not counted):
    17 operands through the padded c2r (x, y, z passes), 10 product sums
    through the padded r2c (z, y, x passes), the streaming source products,
    and the assembly of `overload` sub-lattices for positions and velocities."""
    cs = 2 * prec_bytes
    M, Kz = 3 * n // 2, n // 2 + 1
    S_NK, S_MNK, S_MMK = n * n * Kz * cs, M * n * Kz * cs, M * M * Kz * cs
    S_R = M * M * M * prec_bytes  # padded real field
    S_N = n * n * (n + 2) * prec_bytes  # N-grid
    npart = overload * n ** 3
    out = {
        "conv_xinv": 17 * (S_NK + S_MNK),
        "conv_yinv": 17 * (S_MNK + S_MMK),
        "conv_z": 27 * (S_MMK + S_R),
        "conv_yfwd": 10 * (S_MMK + S_MNK),
        "conv_xfwd": 10 * (S_MNK + S_NK),
        # noise r2c z pass + per sub-lattice and pass the three components' c2r z
        # passes with the lattice readout fused (AoS positions / velocities out)
        "fft_z": 2 * S_N + 2 * overload * (3 * S_N + 3 * n ** 3 * prec_bytes),
        # noise r2c y/x passes, three-component assembly x passes (order sum, A3 x3,
        # PLT table of 4 reals per mode, three outputs), component y passes
        "fft_col": 2 * 2 * S_NK + 2 * overload * ((1 + 3 + 3) * S_NK + (2 * S_NK if plt else 0))
                   + 2 * overload * 3 * 2 * S_NK,
        # source products (7 + 10 + 21 real fields), two order sums (3 in, 1 out), ids
        "pointwise": (7 + 10 + 21) * S_R + 2 * 4 * S_NK + npart * 8,
    }
    return out


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch from
# an ncu capture, per unit of work (M^3 of the padded transform), so that it
# scales to other grid sizes; measured at the bench's N=512
TRAFFIC_PER_UNIT = {
    ("conv_z", 4): (2.971e9 / (768 * 768 * 768), "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,"
                                                 "gpu__time_duration.sum (one pass per launch): the 27 k_zconv_tma "
                                                 "launches of one 3LPT BCC IC at N=512 (M=768), FP32 (17 operand "
                                                 "c2r 2.967 GB, 10 product-sum r2c 2.979 GB per launch), mean"),
}


def traffic_per_launch(kind: str, n: int, prec_bytes: int):
    t = TRAFFIC_PER_UNIT.get((kind, prec_bytes))
    if t is None:
        return None, None
    M = 3 * n // 2
    return t[0] * M * M * M, t[1] + ("" if n == 512 else f", scaled to N={n} by M^3")


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU baseline: whole initial conditions of the oracle port
# ---------------------------------------------------------------------------
# grid of the CPU sample: the bench's workload (3LPT + PLT, BCC, z = 24, the
# same box length per cell) at N = 128, so that one whole IC is a bounded
# amount of host work (about 10 s on 16 cores)
CPU_SAMPLE_N = 128


class PortIC:
    """One whole 3LPT + PLT BCC initial condition of the oracle port (the
    numpy/scipy restatement of the reference, pinned to the reference itself
    by the CPU tests): noise -> phi(1) -> phi(2), phi(3), A(3) by Orszag
    convolutions -> PLT-corrected displacements and velocities on both
    sub-lattices -> positions, velocities, IDs.  The PLT tables (init_D) are
    built once, as the pipeline builds them once per generator."""

    def __init__(self, n: int, threads: int, plt_ng: int = 64):
        import numpy as np  # noqa: F401
        from monofonic_gb300 import ic
        from oracle import lpt_oracle as O
        self.O, self.n, self.threads = O, n, threads
        O.set_fft_workers(threads)
        self.L = WORKLOAD["boxlen"] * n / WORKLOAD["ngrid"]
        cosmo = ic.Cosmology(**COSMO)
        sc = ic.cosmology_scalars(cosmo, WORKLOAD["zstart"])
        p = O.cosmo_parameters(COSMO["Omega_m"], COSMO["Omega_b"], COSMO["h"], COSMO["sigma_8"], COSMO["n_s"])
        self.osc = O.scalars_from(p, sc.Dplus, sc.vfac, sc.pnorm)
        t0 = time.perf_counter()
        self.tables = O.plt_tables(1, plt_ng)
        self.plt_ng = plt_ng
        self.table_s = time.perf_counter() - t0
        self.noise = ic.white_noise(n, 12345)

    def run(self) -> float:
        """seconds for one whole IC"""
        import numpy as np
        O, n, L = self.O, self.n, self.L
        t0 = time.perf_counter()
        f = O.lpt_potentials(self.noise, L, 3, self.osc)
        pos = np.empty((2 * n ** 3, 3))
        vel = np.empty_like(pos)
        for d in range(3):
            fr = O.c2r(O.displacement_k_plt(f, L, d, 3, self.tables, unit=L), n)
            pos[:, d] = O.lattice_positions_component(fr, d, 1, L, L)
            fv = O.c2r(O.displacement_k_plt(f, L, d, 3, self.tables, unit=L, vel=True, vfac=self.osc.vfac), n)
            vel[:, d] = O.lattice_velocities_component(fv, 1, L)
        ids = O.particle_ids(n, 1)
        del pos, vel, ids
        return time.perf_counter() - t0

    def describe(self, ics: int) -> str:
        n = self.n
        return (f"oracle port (numpy/scipy FP64, {self.threads} threads): {ics} whole 3LPT+PLT BCC 2x{n}^3 ICs "
                f"(L={self.L:g} Mpc/h, the 512^3 workload's box per cell), timed end to end; PLT tables built once "
                f"beforehand ({self.plt_ng}^3 mesh, {self.table_s:.1f} s, untimed, as the GPU arm builds them at "
                f"create)")


def cpu_sample(threads: int, n: int = CPU_SAMPLE_N):
    """the port's particles/s on one whole IC (after one untimed IC)"""
    port = PortIC(n, threads)
    port.run()
    t = port.run()
    return {"value": 2 * n ** 3 / t, "unit": UNIT, "cores": threads, "kind": "port", "sample": port.describe(1),
            "seconds_per_ic": t}


def workload_config(n, world):
    """the workload both arms report"""
    return {"workload": (f"3LPT BCC 2x{n}^3 particles, Orszag 3/2 (M={3 * n // 2}), L=1000 Mpc/h, z=24, "
                         "Eisenstein-Hu, seeded N(0,1) noise; FP32-bulk with float-pair (~48-bit) order sum and q+Psi"),
            "plt": True, "l2": "inputs larger than L2 (working set > 16 GB)", "parallelism": f"replicas x{world}"}


def run_reference(args):
    """the reference's CPU path: whole ICs of the oracle port (pinned to the
    reference by the CPU tests; the reference itself builds only where its
    sources are, which the GPU machine does not have), all host threads; one step
    is one whole IC at CPU_SAMPLE_N"""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.ref_ngrid
    port = PortIC(n, threads, args.ref_plt_ngrid)
    secs = []
    for i in range(args.warmup + args.steps):
        t = port.run()
        if i >= args.warmup:
            secs.append(t)
    total = sum(secs)
    v = 2 * n ** 3 * args.steps / total
    desc = port.describe(args.steps)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": _launched_world(), "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(WORKLOAD["ngrid"], 1) | {"reference_sample": f"2x{n}^3 per step"},
            "impl": "reference",
            "cpu_baseline": {"kind": "port", "cores": threads, "sample": desc, "value": v, "unit": UNIT},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# batched realizations and the IC server
# ---------------------------------------------------------------------------
BATCH_SIZES = (64, 96, 128, 192, 256)
SERVE_SIZES = (64, 128, 192, 256, 384)


def _draw_cosmology(rng):
    from monofonic_gb300 import ic
    return ic.Cosmology(Omega_m=float(rng.uniform(0.25, 0.35)), Omega_b=COSMO["Omega_b"], h=COSMO["h"],
                        sigma_8=float(rng.uniform(0.7, 0.9)), n_s=float(rng.uniform(0.92, 1.0)))


def _draw_request(rng, sizes, prec):
    from monofonic_gb300.serve import Request
    n = int(rng.choice(sizes))
    return Request(ngrid=n, boxlen=2.0 * n, zstart=WORKLOAD["zstart"], lpt_order=int(rng.choice([2, 3])),
                   lattice="sc", precision=prec, cosmology=_draw_cosmology(rng), seed=int(rng.integers(1, 2 ** 62)))


def _tuning_summary(report: str) -> dict:
    """{"conv_xinv L=768 f32": "occ 0", ...} from an autotuner report"""
    out = {}
    for line in report.splitlines():
        if ":" in line and "->" in line:
            out[line.split(":")[0]] = line.split("->")[1].strip()
    return out


def _pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, max(0, int(math.ceil(q * len(xs))) - 1))]


def run_output(ctx, sc, noise_h, n):
    """GRAFIC-2 output of the 3LPT SC n^3 fields (src/plugins/output_grafic2.cc
    driven by ic_generator.cc:794-891): the pipeline in field mode plus six
    component files, against a plain write() of the same bytes from page-locked
    memory into the same directory (the host's file-write ceiling)."""
    import shutil
    import numpy as np
    from monofonic_gb300 import ic
    from monofonic_gb300.output import Grafic2Output
    d = tempfile.mkdtemp(prefix="mf_grafic2_")
    try:
        cosmo = ic.Cosmology(**COSMO)
        w = Grafic2Output(ctx, os.path.join(d, "ics"), n, WORKLOAD["boxlen"], WORKLOAD["zstart"], 100.0 * COSMO["h"],
                          COSMO["Omega_m"], 1.0 - COSMO["Omega_m"], COSMO["Omega_b"])
        cfg = ic.ICConfig(ngrid=n, boxlen=WORKLOAD["boxlen"], zstart=WORKLOAD["zstart"], lpt_order=3, lattice="sc",
                          precision="f32", out_kind="fields", lunit=w.position_unit(), vunit=w.velocity_unit())
        gen = ic.ICGenerator(ctx, cfg, sc)
        gen.set_noise(noise_h)
        w.write_ic(gen)  # warm-up: pipeline, page cache, staging
        gen.set_noise(noise_h)  # a run consumes the uploaded noise
        t0 = time.perf_counter()
        w.write_ic(gen)
        total_ms = (time.perf_counter() - t0) * 1e3
        lw = w.last_write()
        gen.close()
        w.close()
        # host ceiling: the same bytes written with write() from one 64 MiB page-locked buffer
        chunk = 64 << 20
        pb = ic.PinnedBuffer(chunk)
        buf = pb.array(np.uint8, (chunk,))
        buf[:] = 1
        best = 1e30
        for _ in range(2):
            fn = os.path.join(d, "plain.bin")
            t0 = time.perf_counter()
            fd = os.open(fn, os.O_WRONLY | os.O_CREAT | os.O_TRUNC, 0o644)
            left = lw["bytes"]
            while left > 0:
                left -= os.write(fd, memoryview(buf)[:min(chunk, left)])
            os.close(fd)
            best = min(best, time.perf_counter() - t0)
            os.unlink(fn)
        pb.close()
        host_gbs = lw["bytes"] / best / 1e9
        write_gbs = lw["bytes"] / (lw["wall_ms"] / 1e3) / 1e9
        n3 = n ** 3
        # transpose kernel: 8 B read (float64 field) + 4 B written per cell and component
        kern_gbs = 6 * n3 * 12 / (lw["kernel_ms"] / 1e3) / 1e9 if lw["kernel_ms"] > 0 else None
        return {"format": "grafic2 (RAMSES)", "workload": f"3LPT SC {n}^3 FP32-bulk fields, 6 components",
                "bytes": lw["bytes"], "ic_plus_write_ms": round(total_ms, 1), "write_ms": round(lw["wall_ms"], 1),
                "write_GBps": round(write_gbs, 2), "host_plain_write_GBps": round(host_gbs, 2),
                "frac_of_host_write": round(write_gbs / host_gbs, 3),
                "transpose_kernel_ms": round(lw["kernel_ms"], 2),
                "transpose_kernel_GBps": round(kern_gbs, 1) if kern_gbs else None}
    except Exception as ex:  # an output failure must not break the line
        return {"format": "grafic2 (RAMSES)", "failed": str(ex)}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def run_batch(args, device):
    """Ragged batch of realizations recorded into one CUDA graph: N drawn from
    {64,96,128,192,256}, L = 2N Mpc/h, 2LPT or 3LPT (p = 1/2), per-item seed
    and cosmology (Omega_m U(.25,.35), sigma8 U(.7,.9), n_s U(.92,1)), FP32.
    Each timed step draws new seeds and cosmologies (host cosmology on all
    threads, timed separately) and replays the graph."""
    import numpy as np
    from monofonic_gb300.serve import Batch
    rng = np.random.default_rng(2024)
    reqs = [_draw_request(rng, BATCH_SIZES, "f32") for _ in range(args.batch_items)]
    t0 = time.perf_counter()
    b = Batch(reqs, nstreams=args.batch_streams, device=device, autotune=not args.no_autotune)
    t_create = time.perf_counter() - t0
    tuning = _tuning_summary(b.tuning)
    info = b.info()
    for _ in range(max(3, args.warmup)):
        b.run()
    dev_ms, host_ms = [], []
    for _ in range(args.steps):
        cos = [_draw_cosmology(rng) for _ in reqs]
        seeds = [int(rng.integers(1, 2 ** 62)) for _ in reqs]
        h0 = time.perf_counter()
        b.set_items(0, cos, seeds)
        host_ms.append((time.perf_counter() - h0) * 1e3)
        dev_ms.append(b.run())
    b.close()
    npart = sum(r.npart for r in reqs)
    ms = statistics.median(dev_ms)
    return {"workload": (f"{len(reqs)} realizations, N in {{64,96,128,192,256}}, L=2N Mpc/h, 2LPT/3LPT p=0.5, "
                         "SC, per-item seed and cosmology, FP32-bulk, noise generated on the device"),
            "sizes": {str(n): sum(r.ngrid == n for r in reqs) for n in BATCH_SIZES},
            "lpt3": sum(r.lpt_order == 3 for r in reqs), "particles": npart,
            "streams": args.batch_streams, "graph_launches_per_batch": 1,
            "graph_nodes": info["graph_nodes"], "kernels_per_batch": info["kernels"],
            "device_GB": round(info["device_bytes"] / 1e9, 2), "create_s": round(t_create, 2),
            "ms_per_batch": ms, "ms_per_batch_max": max(dev_ms),
            "realizations_per_s": len(reqs) / (ms / 1e3), "particles_per_s": npart / (ms / 1e3),
            "host_cosmology_ms": statistics.median(host_ms),
            "autotuned_schedules": tuning}


def run_serve(args, device, prec, seconds):
    """Poisson stream of IC requests (rate args.serve_rate /s) for `seconds`:
    N from {64,128,192,256,384}, L = 2N, 2LPT/3LPT p = 1/2, random seed and
    cosmology; admission by device footprint; particles streamed to a counting
    output callback in page-locked chunks.  The pool is warmed with one
    request of every shape first."""
    import numpy as np
    from monofonic_gb300.serve import Server, Request
    rng = np.random.default_rng(7 if prec == "f32" else 8)
    srv = Server(nworkers=args.serve_workers, output="count", device=device)
    for n in SERVE_SIZES:
        for o in (2, 3):
            srv.submit(Request(ngrid=n, boxlen=2.0 * n, zstart=WORKLOAD["zstart"], lpt_order=o, precision=prec))
    srv.drain(600.0)
    nwarm = srv.stats()["submitted"]
    ids, npart = [], 0
    start = time.perf_counter()
    t_next = start
    while t_next - start < seconds:
        dt = t_next - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        r = _draw_request(rng, SERVE_SIZES, prec)
        ids.append(srv.submit(r))
        npart += r.npart
        t_next += float(rng.exponential(1.0 / args.serve_rate))
    drained = True
    try:
        srv.drain(max(120.0, 4 * seconds))
    except Exception:
        drained = False
    res = [srv.wait(i, 0.0) for i in ids] if drained else []
    st = srv.stats()
    srv.close()
    if not res:
        return {"precision": prec, "requests": len(ids), "drained": False, "stats": st}
    lat = [(r["t_done"] - r["t_submit"]) * 1e3 for r in res]
    lat_gpu = [(r["t_gpu_done"] - r["t_submit"]) * 1e3 for r in res]
    wait = [(r["t_admit"] - r["t_submit"]) * 1e3 for r in res]
    span = max(r["t_done"] for r in res) - min(r["t_submit"] for r in res)
    ok = sum(r["status"] == 0 for r in res)
    # service capacity: completions over the span in which the server was busy;
    # an arrival rate above it makes the queue (and p99) grow with the window
    busy = max(r["t_done"] for r in res) - min(r["t_admit"] for r in res)
    capacity = ok / busy if busy > 0 else None
    overloaded = bool(capacity is not None and capacity < 0.95 * args.serve_rate)
    return {"precision": prec, "arrival_rate_per_s": args.serve_rate, "window_s": seconds, "requests": len(ids),
            "capacity_req_per_s": round(capacity, 2) if capacity else None, "overloaded": overloaded,
            "completed": ok, "warmup_requests": nwarm, "workers": args.serve_workers,
            "latency_ms": {"p50": _pct(lat, 0.5), "p99": _pct(lat, 0.99), "max": max(lat)},
            "latency_to_device_done_ms": {"p50": _pct(lat_gpu, 0.5), "p99": _pct(lat_gpu, 0.99)},
            "queue_wait_ms": {"p50": _pct(wait, 0.5), "p99": _pct(wait, 0.99)},
            "particles_per_s": npart / span, "requests_per_s": len(ids) / span,
            "gpu_ms_mean": statistics.mean(r["gpu_ms"] for r in res),
            "peak_device_GB": round(st["peak_bytes"] / 1e9, 2), "pooled_pipelines": st["pooled_pipelines"]}


def run_serve_replicas(args, job, device, prec, seconds):
    """the same Poisson stream served by every rank's GPU from one shared
    queue (replicas.ClaimQueue on the job's store): rank 0 pushes the
    arrivals, each rank claims requests while fewer than 2 x workers of its own
    are in flight and serves them with its own server; latencies are measured
    from the push (one machine, one clock)"""
    import json
    import threading
    import numpy as np
    import torch.distributed as dist
    from monofonic_gb300 import ic as _ic
    from monofonic_gb300.replicas import ClaimQueue
    from monofonic_gb300.serve import Server, Request
    q = ClaimQueue(dist.distributed_c10d._get_default_store(), prefix=f"serve_{prec}")
    srv = Server(nworkers=args.serve_workers, output="count", device=device)
    for n in SERVE_SIZES:
        for o in (2, 3):
            srv.submit(Request(ngrid=n, boxlen=2.0 * n, zstart=WORKLOAD["zstart"], lpt_order=o, precision=prec))
    srv.drain(600.0)
    job.barrier()
    feeder = None
    if job.rank == 0:
        rng = np.random.default_rng(7 if prec == "f32" else 8)

        def feed():
            start = time.time()
            t_next = start
            while t_next - start < seconds:
                dt = t_next - time.time()
                if dt > 0:
                    time.sleep(dt)
                r = _draw_request(rng, SERVE_SIZES, prec)
                q.push(json.dumps({"n": r.ngrid, "o": r.lpt_order, "seed": r.seed, "t": time.time(),
                                   "cos": [r.cosmology.Omega_m, r.cosmology.sigma_8, r.cosmology.n_s]}))
                t_next += float(rng.exponential(1.0 / args.serve_rate))
            q.close_input()
        feeder = threading.Thread(target=feed)
        feeder.start()
    mine, lat, inflight = 0, [], {}

    def reap():
        for rid in list(inflight):
            if srv.poll(rid) is not None:
                lat.append((time.time() - inflight.pop(rid)) * 1e3)

    while True:
        while len(inflight) >= 2 * args.serve_workers:
            reap()
            time.sleep(0.0005)
        c = q.claim(timeout_s=max(120.0, 4 * seconds))
        if c is None:
            break
        d = json.loads(c[1])
        cos = _ic.Cosmology(Omega_m=d["cos"][0], Omega_b=COSMO["Omega_b"], h=COSMO["h"], sigma_8=d["cos"][1],
                            n_s=d["cos"][2])
        rid = srv.submit(Request(ngrid=d["n"], boxlen=2.0 * d["n"], zstart=WORKLOAD["zstart"], lpt_order=d["o"],
                                 lattice="sc", precision=prec, cosmology=cos, seed=d["seed"]))
        inflight[rid] = d["t"]
        mine += 1
    while inflight:
        reap()
        time.sleep(0.0005)
    if feeder is not None:
        feeder.join()
    srv.close()
    total = job.sum_over_ranks(float(mine))
    return {"precision": prec, "arrival_rate_per_s": args.serve_rate, "window_s": seconds, "requests": int(total),
            "replicas": job.world, "served_by_rank0": mine,
            "latency_ms": {"p50": job.max_over_ranks(_pct(lat, 0.5) if lat else 0.0),
                           "p99": job.max_over_ranks(_pct(lat, 0.99) if lat else 0.0),
                           "max": job.max_over_ranks(max(lat) if lat else 0.0)},
            "requests_per_s": total / seconds, "capacity_req_per_s": None, "overloaded": None}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_mf(args):
    import numpy as np
    import torch

    from monofonic_gb300 import replicas

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    job = replicas.init("nccl")  # replicas only: barrier and timing reductions, no data-path collective
    world, rank, local = job.world, job.rank, job.local
    barrier = job.barrier
    max_over_ranks = job.max_over_ranks

    import monofonic_gb300 as mf
    from monofonic_gb300 import ic

    n = args.ngrid
    ctx = mf.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    cosmo = ic.Cosmology(**COSMO)
    sc = ic.cosmology_scalars(cosmo, WORKLOAD["zstart"])
    seed = 12345 + 1000 * rank
    noise_h = ic.white_noise(n, seed)
    noise_d = torch.from_numpy(noise_h).to(torch.device("cuda", local))
    torch.cuda.synchronize()

    def make(prec):
        cfg = ic.ICConfig(ngrid=n, boxlen=WORKLOAD["boxlen"], zstart=WORKLOAD["zstart"],
                          lpt_order=WORKLOAD["lpt_order"], lattice=WORKLOAD["lattice"], precision=prec,
                          lunit=WORKLOAD["boxlen"], vunit=WORKLOAD["boxlen"], pos64=(prec == "f64"), id64=True,
                          plt=True)
        return ic.ICGenerator(ctx, cfg, sc)

    def timed(gen, steps, warmup, clocks=None, profile=False):
        for _ in range(warmup):
            gen.set_noise_device(noise_d.data_ptr())
            gen.run(to_host=False)
        barrier()
        torch.cuda.synchronize()
        ctx.synchronize()
        c0 = ctx.launch_counts()
        if profile:
            ctx.profile(True)
        if clocks:
            clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        per = []
        e0.record(stream)
        for _ in range(steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gen.set_noise_device(noise_d.data_ptr())
            gen.run(to_host=False)
            b.record(stream)
            per.append((a, b))
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.synchronize()
        clk = clocks.stop() if clocks else None
        prof = ctx.profile_read() if profile else None
        if profile:
            ctx.profile(False)
        c1 = ctx.launch_counts()
        total_ms = e0.elapsed_time(e1)
        lat = sorted(a.elapsed_time(b) for a, b in per)
        barrier()
        launches = sum(c1[k] - c0[k] for k in c1)
        return total_ms, lat, prof, clk, launches, stage(gen)

    def stage(gen):
        names = ["noise_r2c+phi1", "phi2", "phi3", "A3", "positions", "velocities", "ids", "handoff"]
        return dict(zip(names, [round(x, 3) for x in gen.stage_times()]))

    # ---- schedules chosen by the autotuner (process-wide) ------------------------
    tuned = {}
    if not args.no_autotune:
        tuned["f32"] = _tuning_summary(ic.autotune(ctx, n, "f32"))
        if not args.no_fp64:
            tuned["f64"] = _tuning_summary(ic.autotune(ctx, n, "f64"))

    # ---- FP32-bulk, inputs resident ------------------------------------------
    gen32 = make("f32")
    npart = gen32.npart
    clocks = Clocks(local)
    total_ms, lat, prof, clk, launches, stages32 = timed(gen32, args.steps, args.warmup, clocks, profile=True)
    total_ms = max_over_ranks(total_ms)
    ms_per_step = total_ms / args.steps
    value = world * npart * args.steps / (total_ms / 1e3)

    # roofline of the dominant kernel kind
    dom = max((k for k in prof if k != "pointwise"), key=lambda k: prof[k][0])
    dom_ms, dom_cnt = prof[dom]
    avg_ms = dom_ms / max(dom_cnt, 1)
    alg = algorithmic_bytes_ic(n, 4, overload=2, plt=True)
    steps_prof = args.steps  # the profiled region covers every timed step
    bpl = alg[dom] * steps_prof / max(dom_cnt, 1)  # algorithmic bytes per launch of the dominant kind
    achieved = bpl / (avg_ms / 1e3) / 1e9
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    kinds = {k: {"ms_total": round(v[0], 3), "launches": v[1],
                 "share": round(v[0] / max(sum(x[0] for x in prof.values()), 1e-9), 4),
                 "GB_s": (round(alg[k] * steps_prof / (v[0] / 1e3) / 1e9, 1) if v[0] > 0 and k in alg else None)}
             for k, v in prof.items()}

    # ---- e2e through the C ABI with page-locked host buffers ------------------
    e2e = None
    if not args.no_e2e:
        pin_noise = ic.PinnedBuffer(noise_h.nbytes)
        pin_noise.array(np.float64, noise_h.shape)[...] = noise_h
        pos = ic.PinnedBuffer(gen32.pos_bytes)
        vel = ic.PinnedBuffer(gen32.vel_bytes)
        ids = ic.PinnedBuffer(gen32.id_bytes)
        def e2e_steps(steps, queued):
            """steps ICs, each with its noise uploaded from page-locked host
            memory and its particles copied back into page-locked host
            buffers.  queued: through mf_ic_run_async (a run's particle copies
            overlap the next run's fields, the next noise upload overlaps the
            run before it; mf_ic_wait ends the region after the last copy);
            else one synchronous mf_ic_run per step"""
            barrier()
            ctx.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            w0 = time.perf_counter()
            e0.record(stream)
            for _ in range(steps):
                gen32.set_noise_host_ptr(pin_noise.ptr)
                if queued:
                    gen32.run_into_async(pos.ptr, vel.ptr, ids.ptr)
                else:
                    gen32.run_into(pos.ptr, vel.ptr, ids.ptr)
            gen32.wait()
            e1.record(stream)
            torch.cuda.synchronize()
            ctx.synchronize()
            return max_over_ranks(e0.elapsed_time(e1)), (time.perf_counter() - w0) * 1e3 / steps

        e2e_steps(max(1, args.warmup), True)
        t, wall_ms = e2e_steps(args.steps, True)
        # the part of the last step after its last kernel: its streamed
        # particle copies still in flight (the copy engine runs at the box's
        # pinned-copy rate; the slices become final only in the assembly)
        handoff_tail_ms = gen32.stage_times()[7]
        t_sync, _ = e2e_steps(args.steps, False)
        ids_h = ids.array(np.uint64, (npart,))
        assert ids_h[1] == 2 and ids_h[n ** 3] == 1, "particle IDs wrong after e2e run"
        # the box's raw device-to-host copy rate into page-locked memory, for context
        # (five samples: on shared hosts the link's rate into page-locked
        # memory varies from copy to copy)
        probe = torch.empty(1 << 30, dtype=torch.uint8, device=torch.device("cuda", local))
        rates = []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mf.lib().mf_copy_to_host(pos.ptr, probe.data_ptr(), probe.numel())
            rates.append(round((1 << 30) / (time.perf_counter() - t0) / 1e9, 1))
        del probe
        hp = C.c_size_t()
        mf.lib().mf_host_huge_page_bytes(C.byref(hp))
        e2e = {"value": world * npart * args.steps / (t / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": int(noise_h.nbytes),
               "d2h_bytes_per_step": int(gen32.pos_bytes + gen32.vel_bytes + gen32.id_bytes),
               "ms_per_step": t / args.steps, "wall_ms_per_step": wall_ms,
               "api": "mf_ic_set_noise (host) + mf_ic_run_async per step, mf_ic_wait at the end",
               "sync_ms_per_step": round(t_sync / args.steps, 3),
               "box_d2h_GBps_pinned_1GiB": max(rates), "box_d2h_GBps_samples": rates,
               "host_buffers": (f"mf_host_alloc: {hp.value >> 20} MB transparent huge pages, registered"
                                if hp.value else "mf_host_alloc: cudaHostAlloc"),
               "handoff_tail_ms_last_step": round(handoff_tail_ms, 2)}
        for b in (pin_noise, pos, vel, ids):
            b.close()
    gen32.close()

    # ---- FP64 plain ---------------------------------------------------------------
    fp64 = None
    if not args.no_fp64:
        gen64 = make("f64")
        t64, lat64, prof64, _, _, stages64 = timed(gen64, args.fp64_steps, 1, None, profile=True)
        t64 = max_over_ranks(t64)
        ms64 = t64 / args.fp64_steps
        fp64_tf = ctx.fma_rate("f64")
        fp64 = {"value": world * npart / (ms64 / 1e3), "unit": UNIT, "ms_per_step": ms64,
                "fp64_fma_peak_tflops_measured": fp64_tf,
                "speedup_fp32_bulk_vs_fp64": ms64 / ms_per_step,
                "kernels": {k: {"ms_total": round(v[0], 2), "launches": v[1]} for k, v in prof64.items()},
                "stages_ms": stages64}
        gen64.close()

    cpu = None
    if rank == 0 and not args.no_cpu and world == 1:
        try:
            cpu = cpu_sample(os.cpu_count() or 1)
            cpu.pop("seconds_per_ic", None)
        except Exception as ex:  # the baseline must not break the GPU line
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {ex}"}

    output = None
    if not args.no_output and rank == 0:
        output = run_output(ctx, sc, noise_h, n)

    batch = None
    if not args.no_batch:
        batch = run_batch(args, local)
    serving = None
    if not args.no_serve:
        serve = run_serve if world == 1 else (lambda a, d, p, sec: run_serve_replicas(a, job, d, p, sec))
        serving = {"f32": serve(args, local, "f32", args.serve_seconds)}
        if not args.no_fp64:
            serving["f64"] = serve(args, local, "f64", args.serve_seconds_fp64)

    if rank == 0:
        p50 = lat[len(lat) // 2]
        p99 = lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]
        roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic_per_launch(dom, n, 4)[0],
                "traffic_source": traffic_per_launch(dom, n, 4)[1], "algorithmic_bytes_per_launch": bpl,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback"}
        detail = {"kernels": kinds, "stages_ms": stages32, "autotuned_schedules": tuned or None, "e2e": e2e,
                  "fp64_plain": fp64, "cpu_baseline": cpu, "clocks": clk, "batch": batch, "serving": serving,
                  "output": output, "roofline": roof, "latency_ms": {"p50": p50, "p99": p99}}
        detail_path = write_detail(args, detail)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(n, world),
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "roofline": roof,
            "latency_ms": {"p50": round(p50, 3), "p99": round(p99, 3)},
            "output": _short_output(output),
            "batch": _short_batch(batch),
            "serving": _short_serving(serving),
            "stages_ms": stages32,
            # per kind: GB/s over the IC's algorithmic bytes, fraction of measured HBM, ms per IC
            "kernels": {k: [v["GB_s"], round(v["GB_s"] / peak, 3) if v["GB_s"] else None,
                            round(v["ms_total"] / args.steps, 2)] for k, v in kinds.items()},
            "fp64_plain": _short_fp64(fp64),
            "detail_file": detail_path,
        }
        print(json.dumps(line))
    job.close()
    return 0


def write_detail(args, detail) -> str | None:
    """the full per-kernel, schedule, batch and serving record, too long for
    the one printed line, goes to a side file"""
    path = args.detail
    if path is None:
        path = os.path.join(tempfile.gettempdir(), "bench_detail.json")
    try:
        with open(path, "w") as f:
            json.dump(detail, f, indent=1)
        return path
    except OSError:
        return None


def _short_output(o):
    if not o or "failed" in o:
        return o
    return {k: o[k] for k in ("write_GBps", "host_plain_write_GBps", "frac_of_host_write", "ic_plus_write_ms")}


def _short_batch(b):
    if not b:
        return b
    return {"items": sum(b["sizes"].values()), "ms_per_batch": round(b["ms_per_batch"], 2),
            "particles_per_s": b["particles_per_s"], "realizations_per_s": round(b["realizations_per_s"], 1),
            "graph_launches_per_batch": b["graph_launches_per_batch"], "kernels_per_batch": b["kernels_per_batch"]}


def _short_serving(s):
    if not s:
        return s
    out = {}
    for prec, r in s.items():
        if "latency_ms" not in r:
            out[prec] = r
            continue
        out[prec] = {"window_s": r["window_s"], "rate": r["arrival_rate_per_s"], "requests": r["requests"],
                     "p50_ms": round(r["latency_ms"]["p50"], 1), "p99_ms": round(r["latency_ms"]["p99"], 1),
                     "served_req_per_s": round(r["requests_per_s"], 2),
                     "capacity_req_per_s": r.get("capacity_req_per_s"), "overloaded": r.get("overloaded")}
    return out


def _short_fp64(f):
    if not f:
        return f
    return {"value": f["value"], "ms_per_step": round(f["ms_per_step"], 2),
            "speedup_fp32_bulk_vs_fp64": round(f["speedup_fp32_bulk_vs_fp64"], 2),
            "fp64_fma_peak_tflops_measured": f["fp64_fma_peak_tflops_measured"]}


def _launched_world() -> int:
    """ranks of the job this process belongs to (1 outside a launcher)"""
    return int(os.environ.get("WORLD_SIZE", "1"))


def relaunch_ranks(n: int) -> int:
    """--gpus N > 1 outside a launcher: start N ranks of this command on one
    node (torch.distributed.run, rendezvous on 127.0.0.1) and return the
    launcher's exit status; every rank then reads RANK / WORLD_SIZE /
    LOCAL_RANK from its environment."""
    import socket
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def run_stub(args):
    """the multi-rank bookkeeping of the GPU arm without a GPU: gloo ranks,
    barrier, max-over-ranks timing and the whole-job rate; rank 0 prints the
    line with the real world size"""
    from monofonic_gb300 import replicas
    job = replicas.init("gloo")
    units = 1000.0 * args.steps
    job.barrier()
    t0 = time.perf_counter()
    time.sleep(0.01 * (job.rank + 1))
    dt = job.max_over_ranks(time.perf_counter() - t0)
    rate = job.aggregate_rate(units, dt)
    ranks = job.sum_over_ranks(1.0)
    if job.rank == 0:
        print(json.dumps({"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": job.world, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "none", "data": "synthetic",
                          "impl": "stub", "ranks_joined": int(ranks), "config": {"workload": "stub"}}))
    job.close()
    return 0


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch_ranks(args.gpus)
    if args.impl == "reference":
        return run_reference(args)
    if args.impl == "stub":
        return run_stub(args)
    return run_mf(args)


if __name__ == "__main__":
    sys.exit(main())
