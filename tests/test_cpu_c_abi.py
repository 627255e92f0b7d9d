"""The C ABI from plain C: every public header compiles as C99 with warnings
as errors, and a C program links libmfgpu.so and calls its host entry points
(no GPU needed) with the same results as the Python mirror."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "monofonic_gb300")


def test_c_client(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from monofonic_gb300 import build, ic
    if not os.path.exists(os.path.join(LIBDIR, "libmfgpu.so")):
        build.build()
    exe = tmp_path / "probe"
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi_probe.c"), "-o", str(exe), "-L", LIBDIR, "-lmfgpu",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    *version, dplus, pnorm, n0 = r.stdout.split()  # the version string may hold spaces
    sc = ic.cosmology_scalars(ic.Cosmology(), 24.0)
    assert float(dplus) == sc.Dplus and float(pnorm) == sc.pnorm
    assert float(n0) == ic.white_noise(8, 12345, nthreads=1)[0, 0, 0]
