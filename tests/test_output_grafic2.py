"""GRAFIC-2 / RAMSES field output (src/plugins/output_grafic2.cc): the
library's files against the numpy restatement of the format, byte for byte,
and the IC-level write against the oracle's fields."""
import os

import numpy as np
import pytest

from oracle import grafic2_oracle as G
from oracle import lpt_oracle as O
from tests.ic_helpers import setup

# the reference's namelist for dirname "out", GridRes 64, Omega_b 0.0488, no
# baryons, as output_grafic2.cc:249-320 streams it
NAMELIST_OUT_64 = """&RUN_PARAMS
cosmo=.true.
pic=.true.
poisson=.true.
hydro=.false.
nrestart=0
nremap=1
nsubcycle=1,2
ncontrol=1
verbose=.false.
/

&INIT_PARAMS
filetype='grafic'
omega_b=0.0488
initfile(1)='out'
/

&AMR_PARAMS
levelmin=6
levelmax=11
nexpand=1
ngridmax=2000000
npartmax=3000000
/

&REFINE_PARAMS
m_refine=6*8.,
/
"""

COSMO = dict(H0=67.74, Omega_m=0.3099, Omega_DE=0.6901, Omega_b=0.0488)


# -- oracle checks (CPU) -----------------------------------------------------
def test_oracle_namelist_literal():
    assert G.ramses_namelist("out", 64, 0.0488) == NAMELIST_OUT_64
    assert "hydro=.true.\n" in G.ramses_namelist("out", 64, 0.0488, baryons=True)


def test_oracle_file_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    n = 8
    f = rng.standard_normal((n, n, n))
    h = G.header(n, 100.0, 49.0, **{k: COSMO[k] for k in ("H0", "Omega_m", "Omega_DE")})
    p = tmp_path / "ic_poscx"
    p.write_bytes(G.file_bytes(f, h))
    assert p.stat().st_size == 52 + n * (4 * n * n + 8)
    h2, f2 = G.read(str(p))
    assert h2.tobytes() == h.tobytes()
    assert np.array_equal(f2, f.astype(np.float32))
    # plane i of the file holds g(k, j, i) at offset j*n + k
    raw = np.frombuffer(p.read_bytes(), dtype=np.uint8)
    first = raw[52 + 4:52 + 4 + 4 * n * n].view("<f4").reshape(n, n)
    assert np.array_equal(first, f[:, :, 0].T.astype(np.float32))
    assert float(h["dxini0"]) == np.float32(100.0 / 0.6774 / n)
    assert G.file_name("d", "baryon", "vz") == os.path.join("d", "ic_velbz")
    assert G.ignores("dm", "density") and G.ignores("baryon", "dx") and not G.ignores("baryon", "density")


# -- the library on the GPU ----------------------------------------------------
def _writer(ctx, d, n, **kw):
    from monofonic_gb300.output import Grafic2Output
    args = dict(boxlen=100.0, zstart=49.0, **COSMO)
    args.update(kw)
    return Grafic2Output(ctx, str(d), n, **args)


def _hdr(n, boxlen=100.0, zstart=49.0):
    return G.header(n, boxlen, zstart, COSMO["H0"], COSMO["Omega_m"], COSMO["Omega_DE"])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("chunk", [0, 5])
def test_write_grid_bytes(ctx, tmp_path, prec, chunk):
    import monofonic_gb300 as mf
    n = 32
    d = tmp_path / "out"
    w = _writer(ctx, d, n, chunk_planes=chunk)
    assert (d / "ramses.nml").read_text() == G.ramses_namelist(str(d), n, COSMO["Omega_b"])
    rng = np.random.default_rng(11)
    field = rng.standard_normal((n, n, n)) * 3.0
    g = mf.Grid_FFT(ctx, n, 100.0, prec=prec)
    g.set_real(field)
    w.write_grid_data(g, "dm", "vy")
    src = field if prec == "f64" else field.astype(np.float32)
    expect = G.file_bytes(src, _hdr(n))
    assert (d / "ic_velcy").read_bytes() == expect
    lw = w.last_write()
    assert lw["bytes"] == len(expect) and lw["kernel_ms"] > 0
    w.close()


@pytest.mark.gpu
def test_write_field_host_and_device(ctx, tmp_path):
    import torch
    n = 16
    d = tmp_path / "o2"
    w = _writer(ctx, d, n, chunk_planes=3)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((n, n, n))
    w.write_field(f, "baryon", "density")
    assert (d / "ic_deltab").read_bytes() == G.file_bytes(f, _hdr(n))
    t = torch.tensor(f.astype(np.float32), device="cuda")
    torch.cuda.synchronize()
    w.write_field(t.data_ptr(), "neutrino", "vx", prec="f32")
    assert (d / "ic_velnx").read_bytes() == G.file_bytes(f.astype(np.float32), _hdr(n))
    # components the plugin skips write nothing
    w.write_field(f, "dm", "density")
    w.write_field(f, "baryon", "dx")
    w.write_field(f, "baryon", "mass")
    assert not (d / "ic_deltac").exists() and not (d / "ic_posbx").exists() and not (d / "ic_massb").exists()
    w.close()


@pytest.mark.gpu
def test_plugin_queries_and_errors(ctx, tmp_path):
    import monofonic_gb300 as mf
    from monofonic_gb300 import ic
    n = 16
    w = _writer(ctx, tmp_path / "o3", n, ramses_nml=False)
    assert not (tmp_path / "o3" / "ramses.nml").exists()
    assert w.write_species_as("dm") == "field_lagrangian"
    assert w.write_species_as("baryon") == "field_eulerian"
    assert not w.has_64bit_reals() and not w.has_64bit_ids()
    assert w.position_unit() == 100.0 and w.velocity_unit() == 100.0
    assert w.mass_unit() == pytest.approx(1.0 / COSMO["Omega_m"])
    w2 = _writer(ctx, tmp_path / "o4", n, use_spt=True)
    assert w2.write_species_as("baryon") == "field_lagrangian"
    with pytest.raises(mf.MFError, match="power of 2"):
        _writer(ctx, tmp_path / "o5", 48)
    # pipeline in particle mode, or with units other than the plugin's
    cosmo, sc, _ = setup(49.0)
    gp = ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=100.0, zstart=49.0, lpt_order=1, lunit=100.0,
                                         vunit=100.0), sc)
    gp.set_noise(ic.white_noise(n, 1))
    with pytest.raises(mf.MFError, match="MF_OUT_FIELDS"):
        w.write_ic(gp)
    gu = ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=100.0, zstart=49.0, lpt_order=1, out_kind="fields"), sc)
    gu.set_noise(ic.white_noise(n, 1))
    with pytest.raises(mf.MFError, match="units"):
        w.write_ic(gu)
    # a grid still in k-space
    g = mf.Grid_FFT(ctx, n, 100.0, space="k")
    with pytest.raises(mf.MFError, match="real space"):
        w.write_grid_data(g, "dm", "dx")
    for o in (gp, gu, w, w2):
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ic_write_grafic2(ctx, tmp_path, prec):
    """ic_generator.cc:794-891 with the grafic2 plugin: six files of the dark
    matter displacements and velocities in the plugin's units"""
    from monofonic_gb300 import ic
    n, L, z = 32, 100.0, 24.0
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, 99)
    d = tmp_path / "ics"
    w = _writer(ctx, d, n, boxlen=L, zstart=z)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=3, precision=prec, out_kind="fields",
                      lunit=w.position_unit(), vunit=w.velocity_unit())
    gen = ic.ICGenerator(ctx, cfg, sc)
    gen.set_noise(noise)
    w.write_ic(gen)
    lw = w.last_write()
    assert lw["bytes"] == 6 * (52 + n * (4 * n * n + 8))
    # byte-exact against the format applied to the pipeline's own fields
    gen.set_noise(noise)  # a run consumes the uploaded noise
    pos, vel, _ = gen.run()
    hdr = _hdr(n, L, z)
    names = ["dx", "dy", "dz", "vx", "vy", "vz"]
    for k, c in enumerate(names):
        src = (pos if k < 3 else vel)[k % 3]
        assert open(G.file_name(str(d), "dm", c), "rb").read() == G.file_bytes(src, hdr), c
    # and against the oracle's fields, to float rounding (FP64) / the FP32-bulk bound
    f = O.lpt_potentials(noise, L, 3, osc)
    for k, c in enumerate(names):
        r = O.c2r(O.displacement_k(f, L, k % 3, 3, unit=L, vel=k >= 3, vfac=osc.vfac), n)
        h, got = G.read(G.file_name(str(d), "dm", c))
        assert int(h["n1"]) == n
        err = np.linalg.norm(got.astype(np.float64) - r) / np.linalg.norm(r)
        assert err < (1e-7 if prec == "f64" else 1e-5), (c, err)
    gen.close()
    w.close()
