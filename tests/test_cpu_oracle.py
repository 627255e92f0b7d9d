"""CPU tests: the oracle against published known-answer vectors and its own
invariants, the host-side C++ of libmfgpu against the oracle, and the C ABI's
exported symbols.  No GPU is touched."""
import math
import os
import re

import numpy as np
import pytest

from oracle import lpt_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# -- Philox4x32-10 known-answer vectors (Salmon et al. 2011, Random123) -------
@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_kat(ctr, key, expect):
    out = O.philox4x32([np.array([c], dtype=np.uint64) for c in ctr], key)
    assert [int(o[0]) for o in out] == expect


def test_white_noise_statistics():
    x = O.white_noise(32, 12345)
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1) < 0.01
    assert not np.array_equal(x, O.white_noise(32, 12346))


def test_fft_roundtrip_and_unitarity():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((12, 12, 12))
    X = O.r2c(x)
    assert np.allclose(O.c2r(X, 12), x, atol=1e-13)
    # unitary: sum |x|^2 = sum_k w |X|^2 over the half spectrum
    w = np.ones(X.shape); w[:, :, 1:6] = 2
    assert math.isclose(np.sum(x * x), np.sum(w * np.abs(X) ** 2), rel_tol=1e-12)


def test_orszag_dealiases_quadratic_product():
    """Orszag 3/2 padding makes the product of two band-limited fields exact
    on the retained modes (convolution.hh:429-669)."""
    n, L = 16, 1.0
    i = np.arange(n)
    xx = np.meshgrid(i, i, i, indexing="ij")
    f = np.cos(2 * np.pi * 3 * xx[0] / n) + np.sin(2 * np.pi * 2 * xx[1] / n)
    g = np.cos(2 * np.pi * 4 * xx[2] / n)
    got = O.c2r(O.orszag_conv2(O.r2c(f), O.r2c(g)), n)
    assert np.allclose(got, f * g, atol=1e-12)


def test_particle_ids_layout():
    ids = O.particle_ids(4, 1)
    assert ids[0] == 0 and ids[1] == 2 and ids[64] == 1 and ids[65] == 3
    assert len(np.unique(ids)) == 128


def test_power_spectrum_of_white_noise():
    n, L = 32, 100.0
    X = O.r2c(O.white_noise(n, 7))
    k, P, eP, c = O.power_spectrum(X, L)
    # unit-variance white noise: P = (L/n)^3 / (2pi)^3 * n^3 / n^3 ... flat
    flat = P[c > 50]
    assert np.std(flat) / np.mean(flat) < 0.2


# -- host-side C++ of libmfgpu (no device calls) -------------------------------
@pytest.fixture(scope="module")
def mflib():
    from monofonic_gb300 import build
    if not os.path.exists(os.path.join(ROOT, "monofonic_gb300", "libmfgpu.so")):
        build.build()
    import monofonic_gb300 as mf
    return mf.lib()


def test_abi_exports_every_declared_symbol(mflib):
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:int|void|double|const char\s*\*)\s+(mf_\w+)\s*\(", txt, re.M))
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(mflib, n)]
    assert not missing, missing


def test_host_cosmology_matches_oracle(mflib):
    from monofonic_gb300 import ic
    for (om, s8, ns, z) in [(0.3099, 0.8102, 0.9667, 49.0), (0.27, 0.75, 0.95, 24.0)]:
        c = ic.Cosmology(Omega_m=om, sigma_8=s8, n_s=ns)
        s = ic.cosmology_scalars(c, z)
        p = O.cosmo_parameters(om, 0.0488, 0.6774, s8, ns)
        ref = O.cosmo_calculator(p, z)
        assert math.isclose(s.Dplus, ref.Dplus, rel_tol=1e-12)
        assert math.isclose(s.vfac, ref.vfac, rel_tol=1e-12)
        assert math.isclose(s.pnorm, ref.pnorm, rel_tol=1e-9)
        k = np.logspace(-4, 3, 50)
        assert np.allclose(ic.eh_transfer(c, k), O.EisensteinHu(p).at_k(k), rtol=1e-14, atol=0)


def test_host_noise_matches_oracle(mflib):
    from monofonic_gb300 import ic
    for n in (8, 16, 33 - 1):
        a = ic.white_noise(n, 2024, nthreads=3)
        assert np.allclose(a, O.white_noise(n, 2024), rtol=1e-14, atol=1e-14)


def test_host_noise_golden_fixture(mflib):
    """the project RNG plugin reproduces the committed field bit for bit, on
    any thread count, and agrees with the oracle's libm restatement"""
    from monofonic_gb300 import ic
    ref = np.load(os.path.join(ROOT, "tests", "golden", "noise_n16_seed12345.npy"))
    for nt in (1, 4):
        assert np.array_equal(ic.white_noise(16, 12345, nthreads=nt), ref)
    assert np.allclose(ref, O.white_noise(16, 12345), rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("name", ["lpt3_bcc_n16", "lpt2_sc_naive_fixinv_n16", "fields_baryons_eulerian_lpt2_sc_n16"])
def test_oracle_reproduces_the_reference_fixture(mflib, name):
    """the reference's own output (tests/golden/ref_<case>.npz, written by
    tests/golden/make_ref_fixtures.py from oracle/_ref) is what the oracle
    computes from the same noise and scalars, to 1e-12; runs without the
    reference's sources"""
    from tests import ref_cases as R
    case, scalars, want = R.load_fixture(name)
    got = R.to_fixture_keys(case, R.oracle_outputs(case, scalars))
    for key, w in want.items():
        if key.endswith("_pk"):
            continue
        g = got[key]
        if w.dtype.kind in "ui":
            assert np.array_equal(g.astype(w.dtype), w), key
        else:
            assert np.linalg.norm(g - w) / np.linalg.norm(w) < 1e-12, key


# -- further invariants of the oracle ----------------------------------------
def test_inverse_laplacian_inverts_the_laplacian():
    """apply_InverseLaplacian (grid_fft.hh:440-449) undoes -k^2 except on the
    zeroed DC mode"""
    n, L = 16, 50.0
    X = O.r2c(np.random.default_rng(2).standard_normal((n, n, n)))
    kx, ky, kz = O.kgrids(n, L)
    Y = O.inverse_laplacian(-(kx * kx + ky * ky + kz * kz) * X, L)
    X0 = X.copy()
    X0[0, 0, 0] = 0
    assert Y[0, 0, 0] == 0 and np.allclose(Y, X0, rtol=1e-13, atol=1e-13)


def test_shift_field_by_whole_cells_is_a_roll():
    """shift_field (grid_fft.hh:832-842): a shift by whole cells moves the
    field on the grid; a shift and its inverse restore it"""
    n, L = 16, 50.0
    x = np.random.default_rng(3).standard_normal((n, n, n))
    assert np.allclose(O.shift_field(x, (1.0, 0.0, 2.0), L), np.roll(x, (-1, -2), axis=(0, 2)), atol=1e-12)
    # the Nyquist planes of a half-cell shift lose their imaginary parts: compare band-limited fields
    X = O.r2c(x)
    X[n // 2] = 0
    X[:, n // 2] = 0
    X[:, :, n // 2] = 0
    xb = O.c2r(X, n)
    back = O.shift_field(O.shift_field(xb, (0.5, 0.25, -0.5), L), (-0.5, -0.25, 0.5), L)
    assert np.allclose(back, xb, atol=1e-12)


@pytest.mark.parametrize("lattice", [0, 1, 2, 3])
def test_particle_ids_are_a_permutation(lattice):
    """particle IDs of each lattice (particle_generator.hh:212-253): overload*cell + iload,
    every ID exactly once, sub-lattice s occupying particles s*n^3 .. (s+1)*n^3-1"""
    n = 8
    overload = 1 << lattice
    ids = O.particle_ids(n, lattice)
    assert len(ids) == overload * n ** 3
    assert np.array_equal(np.sort(ids), np.arange(overload * n ** 3, dtype=ids.dtype))
    for s in range(overload):
        assert np.all(ids[s * n ** 3:(s + 1) * n ** 3] % overload == s)
    assert np.array_equal(O.particle_ids(n, lattice, id_offset=1) - ids, np.full(len(ids), overload * n ** 3))


def test_naive_and_orszag_agree_on_band_limited_products():
    """for fields whose product stays inside the grid's band the aliased
    (NaiveConvolver) and dealiased (OrszagConvolver) products coincide"""
    n = 16
    i = np.arange(n)
    xx = np.meshgrid(i, i, i, indexing="ij")
    f = np.cos(2 * np.pi * 2 * xx[0] / n) + np.sin(2 * np.pi * 1 * xx[2] / n)
    g = np.cos(2 * np.pi * 3 * xx[1] / n)
    A, B = O.r2c(f), O.r2c(g)
    assert np.allclose(O.naive_conv2(A, B), O.orszag_conv2(A, B), atol=1e-12)
    h = np.sin(2 * np.pi * 1 * xx[0] / n)
    C3 = O.r2c(h)
    assert np.allclose(O.c2r(O.orszag_conv3(A, B, C3), n), f * g * h, atol=1e-12)
