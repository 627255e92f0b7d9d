"""Build libmfgpu.so in-tree for sm_103a.

Every .cu/.cpp file under csrc/ is compiled by its own nvcc process (run in
parallel), then linked into monofonic_gb300/libmfgpu.so.  Objects are cached
under monofonic_gb300/_build/, each keyed on a content hash of its source, of
every header it may include, of the compiler flags and of the machine
architecture; the library is relinked when the set of object keys changes.
A copied tree with stale binaries (other machine, other flags, edited
sources with older timestamps) therefore always recompiles what differs.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
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


def _headers_digest():
    """one digest over the contents of every header under csrc/ and include/"""
    h = hashlib.sha256()
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(os.path.dirname(HERE), "include")
    if os.path.isdir(inc):
        paths += [os.path.join(inc, f) for f in os.listdir(inc)]
    for p in sorted(paths):
        h.update(os.path.basename(p).encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _objdir():
    if not EXTRA:
        return BUILD
    return os.path.join(BUILD, hashlib.sha1(" ".join(EXTRA).encode()).hexdigest()[:10])


def _key(src, hdr_digest):
    h = hashlib.sha256()
    with open(os.path.join(CSRC, src), "rb") as f:
        h.update(f.read())
    h.update(hdr_digest.encode())
    h.update(" ".join([*ARCH, *FLAGS, *EXTRA]).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _read(path):
    try:
        with open(path) as f:
            return f.read()
    except OSError:
        return None


def _compile(src, nvcc, hdr_digest, verbose):
    obj = os.path.join(_objdir(), os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    key = _key(src, hdr_digest)
    if os.path.exists(obj) and _read(obj + ".key") == key and not verbose:
        return obj, key, None
    cmd = [nvcc, *ARCH, *FLAGS, *EXTRA, "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-x", "cu", *ARCH, *FLAGS, *EXTRA, "-c", path, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, key, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    if verbose and r.stderr:
        print(r.stderr)
    with open(obj + ".key", "w") as f:
        f.write(key)
    return obj, key, None


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(_objdir(), exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_digest()
    srcs = _sources()
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    objs, keys, errs = [], [], []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for obj, key, err in ex.map(lambda s: _compile(s, nvcc, hdr, verbose), srcs):
            objs.append(obj)
            keys.append(key)
            if err:
                errs.append(err)
    if errs:
        raise RuntimeError("libmfgpu build failed:\n" + "\n".join(errs))
    lib_key = hashlib.sha256("\n".join(keys).encode()).hexdigest()
    stamp = LIB + ".key"
    if not os.path.exists(LIB) or _read(stamp) != lib_key:
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libmfgpu link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(lib_key)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
