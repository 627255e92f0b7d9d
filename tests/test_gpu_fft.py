"""3D r2c/c2r transforms (Grid_FFT::FourierTransformForward/Backward,
src/grid_fft.cc:199-270) against the oracle's unitary numpy transforms."""
import numpy as np
import pytest

from oracle import lpt_oracle as O

pytestmark = pytest.mark.gpu

SIZES = [16, 32, 64, 96, 128, 192]
TOL = {"f64": 1e-13, "f32": 2e-6}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("n", SIZES)
def test_r2c_c2r(ctx, n, prec):
    import monofonic_gb300 as mf
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n, n))
    g = mf.Grid_FFT(ctx, n, 100.0, prec)
    g.set_real(x)
    g.FourierTransformForward()
    X = g.get_k()
    assert rel_l2(X, O.r2c(x)) < TOL[prec]
    g.FourierTransformBackward()
    assert rel_l2(g.get_real(), x) < TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_element_reads(ctx, prec):
    """relem / kelem (grid_fft.hh:179-211) by (i, j, k) and by get_idx read the
    stored layouts element for element"""
    import monofonic_gb300 as mf
    n = 16
    x = np.random.default_rng(3).standard_normal((n, n, n))
    g = mf.Grid_FFT(ctx, n, 100.0, prec)
    g.set_real(x)
    assert g.space == "r" and g.size(3) == n + 2
    assert g.relem(2, 3, 4) == g.get_real()[2, 3, 4]
    assert g.relem(g.get_idx(5, 6, 7)) == x.astype(g.dtype)[5, 6, 7]
    g.FourierTransformForward()
    X = g.get_k()
    assert g.space == "k" and g.size(3) == n // 2 + 1
    assert g.kelem(1, 2, 3) == X[1, 2, 3]
    assert g.kelem(g.get_idx(4, 0, 8)) == X[4, 0, 8]
    with pytest.raises(IndexError):
        g.kelem(n, 0, 0)
    g.close()


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("n", [16, 48 * 2, 128])
def test_c2r_non_hermitian(ctx, n, prec):
    """c2r of a spectrum that is not Hermitian on the kz=0 and kz=n/2 planes:
    FFTW's convention (complex passes on x, y, then c2r along z ignoring the
    imaginary parts of the kz=0 and kz=n/2 terms)."""
    import monofonic_gb300 as mf
    rng = np.random.default_rng(7 + n)
    X = rng.standard_normal((n, n, n // 2 + 1)) + 1j * rng.standard_normal((n, n, n // 2 + 1))
    g = mf.Grid_FFT(ctx, n, 50.0, prec, space="k")
    g.set_k(X)
    g.FourierTransformBackward()
    assert rel_l2(g.get_real(), O.c2r(X, n)) < TOL[prec]


@pytest.mark.gpu
def test_unsupported_size_is_an_error(ctx):
    import monofonic_gb300 as mf
    with pytest.raises(mf.MFError) as e:
        mf.Grid_FFT(ctx, 100, 1.0)
    assert "MF_ERR_SHAPE" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 32, 96])
def test_complex_grid_fft_matches_numpy(ctx, n):
    """Grid_FFT<ccomplex_t> forward/backward (grid_fft.cc:56-63): unitary
    3D complex transforms against numpy's fftn/ifftn"""
    import torch
    import monofonic_gb300 as mf
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))
    t = torch.from_numpy(a.copy()).to("cuda")
    torch.cuda.synchronize()
    assert mf.lib().mf_cgrid_fft(ctx.ptr, t.data_ptr(), n, 0) == 0
    ctx.synchronize()
    ref = np.fft.fftn(a, norm="ortho")
    assert np.linalg.norm(t.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-13
    assert mf.lib().mf_cgrid_fft(ctx.ptr, t.data_ptr(), n, 1) == 0
    ctx.synchronize()
    assert np.linalg.norm(t.cpu().numpy() - a) / np.linalg.norm(a) < 1e-13


@pytest.mark.gpu
def test_power_spectrum_and_its_file(ctx, tmp_path):
    """Compute_PowerSpectrum (grid_fft.cc:1133-1210) against the oracle, and
    Write_PowerSpectrum (grid_fft.cc:1104-1131): header and one line per
    non-empty bin, values in the default stream format (6 significant digits)"""
    import monofonic_gb300 as mf
    n, L = 32, 100.0
    x = O.white_noise(n, 3)
    g = mf.Grid_FFT(ctx, n, L)
    g.set_real(x)
    k, P, eP, c = g.Compute_PowerSpectrum()
    rk, rP, reP, rc = O.power_spectrum(O.r2c(x), L)
    assert np.array_equal(c, rc)
    assert np.allclose(k, rk, rtol=1e-12, atol=0)
    assert np.allclose(P, rP, rtol=1e-10, atol=0)
    assert np.allclose(eP, reP, rtol=1e-8, atol=0)
    path = tmp_path / "input_powerspec.txt"
    g.Write_PowerSpectrum(str(path))
    lines = path.read_text().splitlines()
    assert lines[0] == "# " + "k".rjust(14) + "P(k)".rjust(16) + "err. P(k)".rjust(16) + "#modes".rjust(16)
    rows = np.array([[float(v) for v in ln.split()] for ln in lines[1:]])
    m = c > 0
    assert rows.shape == (m.sum(), 4) and all(len(ln) == 64 for ln in lines[1:])
    assert np.allclose(rows[:, 0], k[m], rtol=1e-5) and np.allclose(rows[:, 1], P[m], rtol=1e-5)
    assert np.array_equal(rows[:, 3].astype(np.int64), c[m])
