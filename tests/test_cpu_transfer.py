"""The CAMB_file transfer plugin (src/plugins/transfer_CAMB_file.cc) as a
host producer of the pipeline's T(k) tables: file format, log-log natural
cubic spline, the low-k clamp, the baryon-CDM combinations, the k^2 table
layout and the sigma_8 normalisation, on a synthetic file whose columns are
the Eisenstein & Hu fit."""
import math

import numpy as np
import pytest

from monofonic_gb300 import ic
from monofonic_gb300.transfer import CAMBTransfer, NaturalCubicSpline


def _write_camb(path, k, dm, extra_bad_row=False):
    with open(path, "w") as f:
        f.write("#    k/h    CDM      baryon   photon   nu    mass_nu  total  no_nu  total_de  Weyl  v_CDM  v_b  v_b-v_c\n")
        for i, kk in enumerate(k):
            row = [kk, dm[i], 0.9 * dm[i], 1.0, 1.0, 0.97 * dm[i], dm[i], 1.0, 1.0, 1.0, 0.5 * dm[i], 0.6 * dm[i], 0.1]
            f.write(" ".join(f"{v:.17e}" for v in row) + "\n")
        if extra_bad_row:
            f.write("1.0 2.0 3.0 4.0 5.0\n")


@pytest.fixture(scope="module")
def camb(tmp_path_factory):
    cosmo = ic.Cosmology()
    k = np.logspace(-5, 2, 600)
    dm = ic.eh_transfer(cosmo, k)
    path = tmp_path_factory.mktemp("camb") / "tf.dat"
    _write_camb(path, k, dm)
    return cosmo, k, dm, CAMBTransfer(str(path))


def test_spline_matches_scipy_natural_spline():
    from scipy.interpolate import CubicSpline
    rng = np.random.default_rng(1)
    x = np.cumsum(rng.uniform(0.1, 1.0, 40))
    y = np.sin(x) + 0.1 * x
    s, ref = NaturalCubicSpline(x, y), CubicSpline(x, y, bc_type="natural")
    xq = np.linspace(x[0], x[-1], 1000)
    assert np.allclose(s(xq), ref(xq), rtol=0, atol=1e-13)
    assert np.allclose(s(x), y, rtol=0, atol=1e-15)
    with pytest.raises(ValueError):
        s(x[-1] + 1e-9)


def test_table_values(camb):
    cosmo, k, dm, tf = camb
    assert tf.kmin == k[1] and tf.kmax == k[-2]
    inner = slice(1, -1)
    assert np.allclose(tf.compute(k[inner]), dm[inner], rtol=1e-13, atol=0)  # through the nodes
    kq = np.logspace(-4.5, 1.5, 777)
    # spline accuracy at 86 nodes per decade (the largest error, 6e-6, on the baryon wiggles)
    assert np.allclose(tf.compute(kq), ic.eh_transfer(cosmo, kq), rtol=2e-5, atol=0)
    # below the second node the plugin clamps k
    assert tf.compute(k[0] * 0.5) == tf.compute(k[1])
    assert np.allclose(tf.compute(k[inner], "delta_bc"), -0.1 * dm[inner], rtol=1e-12)
    assert np.allclose(tf.compute(k[inner], "theta_bc"), 0.1 * dm[inner], rtol=1e-12)
    assert np.allclose(tf.compute(k[inner], "delta_cdm0"), dm[inner], rtol=1e-13)
    assert np.allclose(tf.compute(k[inner], "theta_matter"), dm[inner], rtol=1e-13)
    with pytest.raises(ValueError):
        tf.compute(k[-1] * 1.01)
    with pytest.raises(ValueError):
        tf.compute(1.0, "phi")


def test_pipeline_table_layout(camb):
    _, _, _, tf = camb
    n, L = 64, 100.0
    t = tf.table(n, L)
    assert t.shape == (3 * (n // 2) ** 2 + 1,) and t.dtype == np.float64
    k2 = np.array([0, 1, 2, 3, 1000, 3 * (n // 2) ** 2])
    assert np.array_equal(t[k2], tf.compute(np.sqrt(k2.astype(np.float64)) * (2.0 * math.pi / L)))


def test_sigma8_normalisation(camb):
    """the table of E&H values normalises like the E&H plugin itself"""
    cosmo, _, _, tf = camb
    sc_eh = ic.cosmology_scalars(cosmo, 24.0)
    sc = tf.scalars(cosmo, 24.0)
    assert math.isclose(sc.pnorm, sc_eh.pnorm, rel_tol=1e-4)
    assert sc.Dplus == sc_eh.Dplus and sc.vfac == sc_eh.vfac


def test_malformed_file(tmp_path, camb):
    cosmo, k, dm, _ = camb
    bad = tmp_path / "bad.dat"
    _write_camb(bad, k[:50], dm[:50], extra_bad_row=True)
    with pytest.raises(ValueError):
        CAMBTransfer(str(bad))
    short = tmp_path / "short.dat"
    _write_camb(short, k[:4], dm[:4])
    with pytest.raises(ValueError):
        CAMBTransfer(str(short))
