"""Host-side parameter logic of the C ABI, run without a GPU: the grid sizes
the kernels are built for, the particle container sizes of each lattice
(include/particle_generator.hh:212-253: N^3 times the lattice's overload),
the device footprint the server's admission reads, and the parameter checks
that turn invalid input into an error status before anything is allocated."""
import ctypes as C

import pytest

from monofonic_gb300 import _lib as L
from monofonic_gb300 import ic


@pytest.fixture(scope="module")
def scalars():
    return ic.cosmology_scalars(ic.Cosmology(), 24.0)


def _sizes(cfg, scalars):
    p = cfg.to_c(scalars)
    np_, pb, vb, ib = C.c_int64(), C.c_size_t(), C.c_size_t(), C.c_size_t()
    rc = L.load().mf_ic_output_size(C.byref(p), C.byref(np_), C.byref(pb), C.byref(vb), C.byref(ib))
    return rc, np_.value, pb.value, vb.value, ib.value


def test_grid_sizes():
    lib = L.load()
    for n in (16, 32, 64, 96, 128, 192, 256, 384, 512):
        assert lib.mf_grid_size_supported(n) == 1, n
    for n in (0, 8, 24, 48, 100, 500, 768, 1024):
        assert lib.mf_grid_size_supported(n) == 0, n


@pytest.mark.parametrize("lattice,overload", [("sc", 1), ("bcc", 2), ("fcc", 4), ("rsc", 8)])
@pytest.mark.parametrize("pos64,id64", [(True, True), (False, True), (False, False)])
def test_particle_container_sizes(scalars, lattice, overload, pos64, id64):
    n = 64
    cfg = ic.ICConfig(ngrid=n, boxlen=100.0, zstart=24.0, lattice=lattice, precision="f32", pos64=pos64, id64=id64)
    rc, npart, pb, vb, ib = _sizes(cfg, scalars)
    assert rc == L.MF_OK
    assert npart == overload * n ** 3
    assert pb == vb == 3 * npart * (8 if pos64 else 4)
    assert ib == npart * (8 if id64 else 4)


def test_field_output_sizes(scalars):
    cfg = ic.ICConfig(ngrid=32, boxlen=100.0, zstart=24.0, out_kind="fields")
    rc, npart, pb, vb, ib = _sizes(cfg, scalars)
    assert rc == L.MF_OK and npart == 32 ** 3 and pb == vb == 3 * 8 * 32 ** 3 and ib == 0


def test_footprint_of_the_512_workload(scalars):
    """3LPT+PLT BCC 2x512^3: 22 padded real fields (M=768), three work buffers,
    eight N-grids, the particles and the tabulated PLT gradient"""
    M, n = 768, 512
    for prec, ps, pos64 in (("f32", 4, False), ("f64", 8, True)):
        cfg = ic.ICConfig(ngrid=n, boxlen=1000.0, zstart=24.0, lpt_order=3, lattice="bcc", precision=prec, plt=True,
                          pos64=pos64)
        got = ic.device_footprint(cfg, scalars)
        npart = 2 * n ** 3
        expect = (22 * M ** 3 * ps + 3 * M * M * (n // 2 + 1) * 2 * ps + 8 * (n + 2) * n * n * ps
                  + npart * (6 * (8 if pos64 else 4) + 8) + 4 * n * n * (n // 2 + 1) * ps)
        # plus the k^2 table of the transfer function and other small buffers
        assert expect <= got < expect + 16 * 2 ** 20, (prec, got, expect)
    # the per-term convolutions trade the real fields for two padded work buffers
    cfg = ic.ICConfig(ngrid=n, boxlen=1000.0, zstart=24.0, lpt_order=3, lattice="bcc", precision="f32", plt=True,
                      pos64=False, per_term_conv=True)
    assert ic.device_footprint(cfg, scalars) < 20e9


def test_footprint_grows_with_order_and_size(scalars):
    f = lambda **kw: ic.device_footprint(ic.ICConfig(boxlen=100.0, zstart=24.0, precision="f32", **kw), scalars)
    assert f(ngrid=64, lpt_order=1) < f(ngrid=64, lpt_order=2) < f(ngrid=64, lpt_order=3)
    assert f(ngrid=64, lpt_order=3) < f(ngrid=128, lpt_order=3) < f(ngrid=256, lpt_order=3)


@pytest.mark.parametrize("change,code", [
    (dict(ngrid=100), L.MF_ERR_SHAPE),
    (dict(lpt_order=4), L.MF_ERR_ARG),
    (dict(lpt_order=0), L.MF_ERR_ARG),
    (dict(boxlen=0.0), L.MF_ERR_ARG),
    (dict(out_kind="fields", lattice="bcc"), L.MF_ERR_ARG),
    (dict(plt=True, plt_ngrid=50), L.MF_ERR_SHAPE),
    (dict(baryons=True, munit=0.0), L.MF_ERR_ARG),
])
def test_invalid_parameters_are_refused(scalars, change, code):
    kw = dict(ngrid=32, boxlen=100.0, zstart=24.0)
    kw.update(change)
    cfg = ic.ICConfig(**kw)
    assert _sizes(cfg, scalars)[0] == code
    with pytest.raises(L.MFError) as e:
        ic.device_footprint(cfg, scalars)
    assert e.value.code == code


def test_grid_index_and_wave_vector_helpers():
    """Grid_FFT::size / get_idx / get_k / gradient / laplacian of the Python
    mirror (host arithmetic) against the oracle's per-axis k and gradient"""
    import numpy as np
    import monofonic_gb300 as mf
    from oracle import lpt_oracle as O
    n, L = 16, 100.0
    assert mf.grid_sizes(n, "r") == (16, 16, 16, 18) and mf.grid_sizes(n, "k") == (16, 16, 9, 9)
    k1, g1 = O.kvec_1d(n, L), O.grad_1d(n, L)
    for i in range(n):
        for j in range(0, n, 3):
            for k in range(n // 2 + 1):
                kv = mf.grid_wave_vector(n, L, i, j, k)
                assert np.array_equal(kv, [k1[i], k1[j], k1[k]])
                for d, x in enumerate((i, j, k)):
                    assert mf.grid_gradient(n, L, d, (i, j, k)) == complex(0.0, g1[x])
                assert mf.grid_laplacian(n, L, (i, j, k)) == -(k1[i] ** 2 + k1[j] ** 2 + k1[k] ** 2)
    # FP32 grids compute in float: the same formula in single precision
    kv32 = mf.grid_wave_vector(n, L, 9, 3, 8, np.float32)
    kf = np.float32(2.0 * np.pi / L)
    assert kv32.dtype == np.float32
    assert np.array_equal(kv32, [np.float32(-7) * kf, np.float32(3) * kf, np.float32(8) * kf])
