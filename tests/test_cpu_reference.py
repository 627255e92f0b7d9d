"""Parity pinned to the reference itself: oracle/_ref is the reference's own
monofonIC program compiled from its unmodified sources against the project
shims (oracle/ref/), with the project RNG plugin and a capture output plugin
registered through the reference's plugin interfaces.  These CPU tests check
  * the shims themselves (the FFT against numpy, the computed Gauss-Kronrod
    rule's exactness),
  * the pipeline's host cosmology (mf_cosmology_compute) against the scalars
    the reference computes,
  * the numpy oracle against the reference, case by case (particles, fields,
    two species, PLT, the Eulerian branch, the power spectrum), and
  * that the committed fixtures are what the reference produces.
They need the reference's sources (present in the build container); without
them they are skipped."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import refrun
from tests import ref_cases as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref():
    if not refrun.sources_present() and not refrun.available():
        pytest.skip("the reference's sources are not on this machine (oracle/_ref cannot be built)")
    assert refrun.build(), "oracle/_ref did not build"
    return refrun


def test_fft_shim_matches_numpy(tmp_path):
    """the FFTW3-API shim behind oracle/_ref: r2c, c2r (with FFTW's treatment
    of non-Hermitian kz = 0, n/2 planes) and c2c against numpy, odd and even
    sizes, unnormalised"""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    so = tmp_path / "libfftwshim.so"
    r = subprocess.run([cxx, "-O2", "-std=c++14", "-fopenmp", "-shared", "-fPIC", "-o", str(so),
                        os.path.join(ROOT, "oracle", "ref", "shim", "fftw_shim.cc")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(so))
    for f in ("fftw_plan_dft_r2c_3d", "fftw_plan_dft_c2r_3d"):
        getattr(lib, f).restype = C.c_void_p
        getattr(lib, f).argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_void_p, C.c_uint]
    lib.fftw_plan_dft_3d.restype = C.c_void_p
    lib.fftw_plan_dft_3d.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_void_p, C.c_int, C.c_uint]
    lib.fftw_execute.argtypes = [C.c_void_p]
    lib.fftw_destroy_plan.argtypes = [C.c_void_p]
    rng = np.random.default_rng(0)
    for shp in [(8, 8, 8), (16, 12, 18), (24, 32, 48), (5, 7, 9), (6, 10, 14)]:
        n0, n1, n2 = shp
        nc = n2 // 2 + 1
        x = rng.standard_normal(shp)
        buf = np.zeros((n0, n1, 2 * nc))
        buf[:, :, :n2] = x
        p = lib.fftw_plan_dft_r2c_3d(n0, n1, n2, buf.ctypes.data, buf.ctypes.data, 64)
        lib.fftw_execute(p)
        lib.fftw_destroy_plan(p)
        want = np.fft.rfftn(x)
        got = buf.view(np.complex128)
        assert np.abs(got - want).max() < 1e-14 * np.abs(want).max()
        Y = rng.standard_normal(want.shape) + 1j * rng.standard_normal(want.shape)
        yb = np.ascontiguousarray(Y.copy())
        p = lib.fftw_plan_dft_c2r_3d(n0, n1, n2, yb.ctypes.data, yb.ctypes.data, 64)
        lib.fftw_execute(p)
        lib.fftw_destroy_plan(p)
        want = np.fft.irfftn(Y, s=shp, axes=(0, 1, 2)) * np.prod(shp)
        assert np.abs(yb.view(np.float64)[:, :, :n2] - want).max() < 1e-14 * np.abs(want).max()
        Z = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
        for sign, want in ((-1, np.fft.fftn(Z)), (1, np.fft.ifftn(Z) * np.prod(shp))):
            zb = np.ascontiguousarray(Z.copy())
            p = lib.fftw_plan_dft_3d(n0, n1, n2, zb.ctypes.data, zb.ctypes.data, sign, 64)
            lib.fftw_execute(p)
            lib.fftw_destroy_plan(p)
            assert np.abs(zb - want).max() < 1e-14 * np.abs(want).max()


def test_gauss_kronrod_rule_is_exact(tmp_path):
    """the computed 61-point Gauss-Kronrod rule (mf_quad.h, used by the host
    cosmology and the GSL shim) integrates x^m exactly for m <= 91, its Gauss
    part for m <= 59, and QAG reaches the requested tolerance"""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "gk.cc"
    src.write_text(r'''
#include <cmath>
#include <cstdio>
#include "mf_quad.h"
int main() {
  const mf::quad::GKRule R = mf::quad::make_rule(30);
  double wk = 0, wg = 0;
  for (int m = 0; m <= 91; ++m) {
    double sk = 0, sg = 0;
    for (size_t i = 0; i < R.xk.size(); ++i) { sk += R.wk[i] * std::pow(R.xk[i], m); sg += R.wg[i] * std::pow(R.xk[i], m); }
    const double ex = (m % 2) ? 0.0 : 2.0 / (m + 1);
    wk = std::fmax(wk, std::fabs(sk - ex));
    if (m <= 59) wg = std::fmax(wg, std::fabs(sg - ex));
  }
  double r = 0, e = 0;
  auto f = [](double x) { return std::exp(-x) * std::sin(7 * x); };
  const int st = mf::quad::qag(R, f, 0.0, 20.0, 0.0, 1e-12, 1000, &r, &e);
  const double ex = (7.0 - std::exp(-20.0) * (std::sin(140.0) + 7 * std::cos(140.0))) / 50.0;
  std::printf("%zu %.3e %.3e %d %.3e\n", R.xk.size(), wk, wg, st, std::fabs(r - ex) / ex);
  return 0;
}
''')
    exe = tmp_path / "gk"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "monofonic_gb300", "csrc"), str(src),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    npts, wk, wg, st, rel = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()
    assert int(npts) == 61 and float(wk) < 2e-15 and float(wg) < 2e-15
    assert int(st) == 0 and float(rel) < 1e-12


@pytest.mark.parametrize("cosmo,z", [({}, 24.0), ({}, 49.0), ({"Omega_m": 0.25, "sigma_8": 0.7, "n_s": 0.92}, 30.0),
                                     ({"Omega_m": 0.35, "Omega_b": 0.05, "h": 0.7, "sigma_8": 0.9, "n_s": 1.0}, 99.0)])
def test_host_cosmology_matches_reference(ref, cosmo, z):
    """D+, vfac and pnorm of the pipeline's host calculator equal the
    reference's (cosmology_calculator.hh) to rounding: same growth ODE stepper
    (including its retry from the rejected trial state), log-log splines and
    QAG-61 sigma_8 integral"""
    from monofonic_gb300 import ic
    kw = dict(R.COSMO, **cosmo)
    case = dict(ngrid=16, boxlen=40.0, zstart=z, lpt_order=1, lattice="sc", seed=1, cosmology=kw)
    sc = ref.run(case)["scalars"]
    mine = ic.cosmology_scalars(ic.Cosmology(**kw), z)
    assert abs(mine.Dplus / sc["Dplus"] - 1) < 1e-13
    assert abs(mine.vfac / sc["vfac"] - 1) < 1e-13
    assert abs(mine.pnorm / sc["pnorm"] - 1) < 1e-13


SMALL = [k for k, v in R.CASES.items() if v["ngrid"] <= 64]


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference(ref, name):
    """the numpy oracle restates what the reference hands its output plugin,
    to 1e-12 (rel-L2 of displacements, velocities, masses and fields), IDs
    exact, for the same noise and scalars"""
    case = R.CASES[name]
    res = ref.run(case)
    want = R.to_fixture_keys(case, res)
    got = R.to_fixture_keys(case, R.oracle_outputs(case, res["scalars"]))
    for key in want:
        if key.endswith("_pk"):
            continue
        assert key in got, key
        w, g = want[key], got[key]
        if w.dtype.kind in "ui":
            assert np.array_equal(g.astype(w.dtype), w), key
        else:
            err = float(np.linalg.norm(g - w) / np.linalg.norm(w))
            assert err < 1e-12, (key, err)


def test_power_spectrum_matches_reference(ref):
    """Compute_PowerSpectrum (src/grid_fft.cc:1133-1210) of the IC's SPT
    density, as the reference computes it at full precision, against the
    oracle's estimator on the same field"""
    from oracle import lpt_oracle as O
    case = R.CASES["config1_lpt2_sc_n64_fields"]
    res = ref.run(case)
    pk = res["dm_pk"]
    k, P, eP, cnt = O.power_spectrum(O.r2c(res["dm_density"]), case["boxlen"])
    m = pk[:, 3] > 0
    assert np.array_equal(cnt[m].astype(np.int64), pk[m, 3].astype(np.int64))
    for a, b in ((k[m], pk[m, 0]), (P[m], pk[m, 1]), (eP[m], pk[m, 2])):
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-12


@pytest.mark.parametrize("name", SMALL)
def test_committed_fixture_is_the_reference_output(ref, name):
    """tests/golden/ref_<case>.npz equals a fresh run of the reference"""
    case, scalars, want = R.load_fixture(name)
    assert case == R.CASES[name]
    res = ref.run(case)
    assert res["scalars"] == scalars
    got = R.reduce_outputs(case, res)
    assert sorted(got) == sorted(want)
    for key in want:
        assert np.array_equal(got[key], want[key]), key
