"""Driver of oracle/_ref, the reference's own monofonIC program compiled from
its unmodified sources against the project shims (oracle/ref/Makefile).

TEST INFRASTRUCTURE ONLY: imported by tests/, tests/golden/make_ref_fixtures.py
and nothing in the product.  One `run()` writes a [setup]/[cosmology]/[random]/
[output] configuration file in the reference's own format (example.conf of the
reference), runs the binary in a scratch directory with the project RNG
plugin (PROJECT_PHILOX: the same white noise as the pipeline's generator) and
the capture output plugin, and loads what the reference handed to its output
plugin: particles (positions, velocities, IDs, masses) or Lagrangian /
Eulerian field grids, plus the cosmology scalars it computed and, in field
mode, the power spectrum file it wrote (input_powerspec_sampled_SPT.txt).

The binaries exist only where the reference's sources are (this repository's
build container); GPU tests use fixtures that tests/golden/make_ref_fixtures.py
wrote from them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("MF_REFERENCE_SRC", "/root/reference")
OUT = os.path.join(HERE, "_ref")
BINARIES = {"plain": "monofonIC_ref", "plt": "monofonIC_ref_plt", "naive": "monofonIC_ref_naive"}


def sources_present() -> bool:
    return os.path.isfile(os.path.join(REF_SRC, "src", "ic_generator.cc"))


def build(jobs: int = 0) -> bool:
    """compile oracle/_ref (make -C oracle/ref) when the reference's sources
    are present; True when all binaries exist afterwards"""
    if sources_present() and shutil.which("make") and shutil.which("g++"):
        j = jobs or os.cpu_count() or 4
        r = subprocess.run(["make", "-C", os.path.join(HERE, "ref"), f"REF={REF_SRC}", f"-j{j}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle/_ref build failed:\n" + r.stdout[-4000:] + r.stderr[-4000:])
    return available()


def available() -> bool:
    return all(os.access(os.path.join(OUT, b), os.X_OK) for b in BINARIES.values())


def _yn(b):
    return "yes" if b else "no"


def config_text(case: dict, outdir: str) -> str:
    c = dict(case)
    cos = c.get("cosmology", {})
    lines = [
        "[setup]",
        f"GridRes = {c['ngrid']}",
        f"BoxLength = {c['boxlen']!r}",
        f"zstart = {c['zstart']!r}",
        f"LPTorder = {c.get('lpt_order', 3)}",
        f"DoBaryons = {_yn(c.get('baryons', False))}",
        f"DoBaryonVrel = {_yn(c.get('baryon_vrel', False))}",
        f"DoFixing = {_yn(c.get('fixing', False))}",
        f"DoInversion = {_yn(c.get('inversion', False))}",
        f"ParticleLoad = {c.get('lattice', 'sc')}",
        "",
        "[cosmology]",
        "ParameterSet = none",
        f"Omega_m = {cos.get('Omega_m', 0.3099)!r}",
        f"Omega_b = {cos.get('Omega_b', 0.0488)!r}",
        f"Omega_L = {cos.get('Omega_L', 1.0 - cos.get('Omega_m', 0.3099))!r}",
        f"H0 = {100.0 * cos.get('h', 0.6774)!r}",
        f"sigma_8 = {cos.get('sigma_8', 0.8102)!r}",
        f"n_s = {cos.get('n_s', 0.9667)!r}",
        "transfer = eisenstein",
        "",
        "[random]",
        "generator = PROJECT_PHILOX",
        f"seed = {int(c.get('seed', 12345))}",
        "",
        "[execution]",
        f"NumThreads = {int(c.get('threads', 1))}",
        "",
        "[output]",
        "format = capture",
        f"filename = {outdir}",
        f"capture_type = {c.get('out', 'particles')}",
        f"capture_type_baryon = {c.get('baryon_out', c.get('out', 'particles'))}",
        f"capture_64bit_reals = {_yn(c.get('real64', True))}",
        f"capture_64bit_ids = {_yn(c.get('id64', True))}",
        f"capture_lunit = {float(c.get('lunit', c['boxlen']))!r}",
        f"capture_vunit = {float(c.get('vunit', c['boxlen']))!r}",
        f"capture_munit = {float(c.get('munit', 1.0))!r}",
        "",
    ]
    return "\n".join(lines)


def binary_for(case: dict) -> str:
    if case.get("convolver", "orszag") == "naive":
        return os.path.join(OUT, BINARIES["naive"])
    return os.path.join(OUT, BINARIES["plt" if case.get("plt", False) else "plain"])


def run(case: dict, keep_dir: str | None = None, timeout: float = 3600.0) -> dict:
    """run the reference on `case`; returns {"scalars": {...}, "<species>_<item>":
    array, ..., "pk": (k, P, err, count) when written, "seconds": wall time}"""
    if not available():
        raise RuntimeError("oracle/_ref is not built (needs the reference's sources; oracle.refrun.build())")
    work = keep_dir or tempfile.mkdtemp(prefix="mf_ref_")
    os.makedirs(work, exist_ok=True)
    try:
        out = os.path.join(work, "capture")
        conf = os.path.join(work, "ic.conf")
        with open(conf, "w") as f:
            f.write(config_text(case, out))
        env = dict(os.environ, OMP_NUM_THREADS=str(int(case.get("threads", 1))))
        import time
        t0 = time.perf_counter()
        r = subprocess.run([binary_for(case), conf], cwd=work, capture_output=True, text=True, timeout=timeout,
                           env=env)
        seconds = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}):\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")
        res: dict = {"seconds": seconds}
        sc = {}
        with open(os.path.join(out, "scalars.txt")) as f:
            for line in f:
                k, v = line.split()
                sc[k] = float(v)
        res["scalars"] = sc
        for fn in sorted(os.listdir(out)):
            if fn.endswith(".npy"):
                res[fn[:-4]] = np.load(os.path.join(out, fn))
            elif fn.endswith("_omega.txt"):
                res[fn[:-4]] = float(open(os.path.join(out, fn)).read())
        pk = os.path.join(work, "input_powerspec_sampled_SPT.txt")
        if os.path.exists(pk):
            res["pk"] = np.loadtxt(pk, comments="#", ndmin=2)
        return res
    finally:
        if keep_dir is None:
            shutil.rmtree(work, ignore_errors=True)
