"""The C++ adapter (include/monofonic_gb300.hpp) on the GPU: the
reference-style program tests/cpp_adapter_probe.cpp, linked against
libmfgpu.so, fills, transforms, convolves and reads back grids on the device
and checks every result it can state exactly (element reads, spaces, wave
vectors, error statuses)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "monofonic_gb300")


def test_adapter_program_on_the_device(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "probe"
    # warnings as errors are enforced by the CPU build of the same program (tests/test_cpu_cpp_adapter.py)
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp_adapter_probe.cpp"), "-o", str(exe), "-L", LIBDIR, "-lmfgpu",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
