"""Host logic of the Python Grid_FFT mirror without a GPU: the library is
replaced by a host fake whose grids are numpy buffers, so element reads,
index helpers and the host-mirror functor methods (grid_fft.hh:450-810) are
checked on the CPU."""
import ctypes as C

import numpy as np
import pytest

import monofonic_gb300 as mf
from monofonic_gb300 import _lib as L


class FakeLib:
    """grids in host memory; the device pointer is the buffer's address"""

    def __init__(self):
        self.grids = {}

    @staticmethod
    def _key(p):
        return p.value if hasattr(p, "value") else p

    def mf_ctx_synchronize(self, ctx):
        return L.MF_OK

    def mf_last_error(self, ctx):
        return b""

    def mf_grid_create(self, ctx, n, boxlen, prec, space, out):
        dt = np.float64 if prec == L.MF_PREC_F64 else np.float32
        h = 1000 + len(self.grids)
        self.grids[h] = {"buf": np.zeros((n + 2) * n * n, dt), "space": space}
        out._obj.value = h
        return L.MF_OK

    def mf_grid_destroy(self, p):
        self.grids.pop(self._key(p), None)
        return L.MF_OK

    def mf_grid_info(self, p, n, prec, space, dptr, nbytes):
        g = self.grids[self._key(p)]
        if space is not None:
            space._obj.value = g["space"]
        if dptr is not None:
            dptr._obj.value = g["buf"].ctypes.data
        return L.MF_OK

    def mf_grid_upload(self, p, host, space):
        g = self.grids[self._key(p)]
        C.memmove(g["buf"].ctypes.data, host, g["buf"].nbytes)
        g["space"] = space
        return L.MF_OK

    def mf_grid_download(self, p, host):
        g = self.grids[self._key(p)]
        C.memmove(host, g["buf"].ctypes.data, g["buf"].nbytes)
        return L.MF_OK

    def mf_copy_to_host(self, host, dev, nbytes):
        C.memmove(host, dev, nbytes)
        return L.MF_OK


@pytest.fixture
def fake(monkeypatch):
    lib = FakeLib()
    monkeypatch.setattr(mf, "lib", lambda: lib)
    ctx = mf.Context.__new__(mf.Context)
    ctx.ptr = C.c_void_p(1)
    yield ctx
    ctx.ptr = None


def _grid(ctx, prec, rng, n=16, boxlen=100.0):
    g = mf.Grid_FFT(ctx, n, boxlen, prec)
    g.set_real(rng.standard_normal((n, n, n)))
    return g


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_element_reads_and_indices(fake, prec):
    rng = np.random.default_rng(0)
    g = _grid(fake, prec, rng)
    x = g.get_real()
    assert g.space == "r" and g.size(3) == 18 and g.relem(2, 3, 4) == x[2, 3, 4]
    assert g.relem(g.get_idx(5, 6, 7)) == x[5, 6, 7]
    X = (rng.standard_normal((16, 16, 9)) + 1j * rng.standard_normal((16, 16, 9))).astype(g.cdtype)
    g.set_k(X)
    assert g.space == "k" and g.size(2) == 9 and g.kelem(1, 2, 3) == X[1, 2, 3]
    assert g.kelem(g.get_idx(15, 15, 8)) == X[15, 15, 8]
    with pytest.raises(IndexError):
        g.kelem(16, 0, 0)
    with pytest.raises(TypeError):
        g.get_k(1, 2)
    assert np.array_equal(g.get_k(9, 3, 8), mf.grid_wave_vector(16, 100.0, 9, 3, 8, g.dtype))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_functions_of_the_field(fake, prec):
    rng = np.random.default_rng(1)
    a, b = _grid(fake, prec, rng), _grid(fake, prec, rng)
    k = a._k_arrays()  # the broadcast wave vectors handed to the k-dependent functions
    for i, j, kz in ((9, 3, 8), (0, 15, 0), (8, 8, 4)):
        assert np.array_equal([k[0][i, 0, 0], k[1][0, j, 0], k[2][0, 0, kz]],
                              mf.grid_wave_vector(16, 100.0, i, j, kz, a.dtype))
    # real space: values and cell positions
    xa, xb = a.get_real(), b.get_real()
    pad = a.download_padded()[:, :, 16:].copy()
    a.apply_function_r_dep(lambda x, r: x + r[2])
    assert np.allclose(a.get_real(), xa + (np.arange(16) * (100.0 / 16)).astype(a.dtype)[None, None, :], rtol=0,
                       atol=1e-5)
    assert np.array_equal(a.download_padded()[:, :, 16:], pad) and a.space == "r"
    a.assign_function_of_grids_r(lambda u, v: u - v, b, b)
    assert np.array_equal(a.get_real(), np.zeros((16, 16, 16), a.dtype))
    a.apply_function_r(lambda x: x + 2)
    assert np.array_equal(a.get_real(), np.full((16, 16, 16), 2, a.dtype))
    # k space: values, wave vectors, index triples, several grids
    Xa = (rng.standard_normal((16, 16, 9)) + 1j * rng.standard_normal((16, 16, 9))).astype(a.cdtype)
    Xb = (rng.standard_normal((16, 16, 9)) + 1j * rng.standard_normal((16, 16, 9))).astype(a.cdtype)
    a.set_k(Xa)
    b.set_k(Xb)
    a.apply_function_k_dep(lambda X, kk: X * kk[0])
    assert np.allclose(a.get_k(), Xa * k[0], rtol=1e-6) and a.space == "k"
    a.assign_function_of_grids_kdep(lambda kk, u, v: u * v * kk[1], b, b)
    assert np.allclose(a.get_k(), Xb * Xb * k[1], rtol=1e-5)
    a.assign_function_of_grids_ijk(lambda ijk, u: u * (ijk[0] + ijk[2]), b)
    idx = np.arange(16)[:, None, None] + np.arange(9)[None, None, :]
    assert np.allclose(a.get_k(), Xb * idx, rtol=1e-6)
    a.assign_function_of_grids_k(lambda u: 2 * u, b)
    a.apply_function_k(np.conj)
    assert np.allclose(a.get_k(), np.conj(2 * Xb), rtol=1e-6)
