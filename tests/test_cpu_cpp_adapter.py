"""The C++ adapter (include/monofonic_gb300.hpp) without a GPU: compiled with
warnings as errors against a host fake of the C ABI (tests/cpp_adapter_fake.cpp),
the reference-style calls of tests/cpp_adapter_probe.cpp pass the right
operands, directions, output operators and factors, and read the right
elements; linked against libmfgpu.so on a machine without a GPU, the failure
to create a context surfaces as mfgpu::error."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "monofonic_gb300")
CXXFLAGS = ["-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include")]


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    return cxx


def test_adapter_against_host_fake(tmp_path):
    exe = tmp_path / "probe_fake"
    cmd = [_cxx(), *CXXFLAGS, "-DMF_FAKE_ABI", os.path.join(ROOT, "tests", "cpp_adapter_probe.cpp"),
           os.path.join(ROOT, "tests", "cpp_adapter_fake.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_adapter_links_and_reports_a_missing_device(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tests/test_gpu_cpp_adapter.py runs the adapter on it")
    from monofonic_gb300 import build
    if not os.path.exists(os.path.join(LIBDIR, "libmfgpu.so")):
        build.build()
    exe = tmp_path / "probe"
    cmd = [_cxx(), *CXXFLAGS, os.path.join(ROOT, "tests", "cpp_adapter_probe.cpp"), "-o", str(exe), "-L", LIBDIR,
           "-lmfgpu", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "exception: mf_ctx_create" in r.stdout, r.stdout + r.stderr
