"""Build libmfgpu.so in-tree for sm_103a.

Every .cu/.cpp file under csrc/ is compiled by its own nvcc process (run in
parallel), then linked into monofonic_gb300/libmfgpu.so.  Objects are cached
under monofonic_gb300/_build/ keyed on the source and header timestamps.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
# extra compile definitions (tuning knobs such as -DMF_ZCONV_TMA_MAXR=4); a
# different set builds into its own object directory
EXTRA = os.environ.get("MF_NVCC_FLAGS", "").split()


def _nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    ts = [os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(os.path.dirname(HERE), "include")
    if os.path.isdir(inc):
        ts += [os.path.getmtime(os.path.join(inc, f)) for f in os.listdir(inc)]
    return max(ts) if ts else 0.0


def _objdir():
    if not EXTRA:
        return BUILD
    return os.path.join(BUILD, hashlib.sha1(" ".join(EXTRA).encode()).hexdigest()[:10])


def _compile(src, nvcc, hdr_t, verbose):
    obj = os.path.join(_objdir(), os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), hdr_t):
        return obj, None
    cmd = [nvcc, *ARCH, *FLAGS, *EXTRA, "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-x", "cu", *ARCH, *FLAGS, *EXTRA, "-c", path, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(_objdir(), exist_ok=True)
    nvcc = _nvcc()
    hdr_t = _headers_mtime()
    srcs = _sources()
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    objs, errs = [], []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for obj, err in ex.map(lambda s: _compile(s, nvcc, hdr_t, verbose), srcs):
            objs.append(obj)
            if err:
                errs.append(err)
    if errs:
        raise RuntimeError("libmfgpu build failed:\n" + "\n".join(errs))
    newest = max(os.path.getmtime(o) for o in objs)
    stamp = LIB + ".flags"
    same_flags = os.path.exists(stamp) and open(stamp).read() == " ".join(EXTRA)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest or not same_flags:
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libmfgpu link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(" ".join(EXTRA))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
