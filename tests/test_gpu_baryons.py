"""Two-species ICs (DoBaryons, ic_generator.cc:153-166, :608-948): dark matter
and baryons with their masses, secondary lattice, IDs and the optional
relative-velocity mode, against the oracle on the same noise.
Tolerances: FP64 rel-L2 <= 1e-12, FP32-bulk <= 1e-5."""
import math

import numpy as np
import pytest

from oracle import lpt_oracle as O
from tests.ic_helpers import COSMO_KW, lattice_q, rel_l2, setup

pytestmark = pytest.mark.gpu
O_LAT = {"sc": 0, "bcc": 1, "fcc": 2, "rsc": 3}


def _tables(n, L):
    """smooth stand-ins for a Boltzmann code's T_delta_bc and T_theta_bc (the
    Eisenstein-Hu plugin returns zero for both), as callables of k and as the
    tables the library takes (k = sqrt(k2)*2pi/L)"""
    Tdbc = lambda k: -0.01 * np.exp(-k / 0.7) / (1.0 + (k / 0.05) ** 2) ** 0.5
    Ttbc = lambda k: 0.003 * np.exp(-k / 0.4) / (1.0 + (k / 0.1) ** 2)
    k = np.sqrt(np.arange(3 * (n // 2) ** 2 + 1, dtype=np.float64)) * (2 * math.pi / L)
    return Tdbc, Ttbc, Tdbc(k), Ttbc(k)


def _run(ctx, n, L, z, order, lattice, prec, tables=False, vrel=False, seed=5, munit=2.5):
    from monofonic_gb300 import ic
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, seed)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=order, lattice=lattice, precision=prec, lunit=L, vunit=L,
                      baryons=True, baryon_vrel=vrel, munit=munit)
    Tdbc = Ttbc = tdbc = ttbc = None
    if tables:
        Tdbc, Ttbc, tdbc, ttbc = _tables(n, L)
    g = ic.ICGenerator(ctx, cfg, sc, tk_dbc=tdbc, tk_tbc=ttbc)
    g.set_noise(noise)
    got = g.run_species()
    f = O.lpt_potentials(noise, L, order, osc)
    ref = O.two_species_particles(f, L, order, osc, COSMO_KW["Omega_m"], COSMO_KW["Omega_b"], lattice=O_LAT[lattice],
                                  lunit=L, vunit=L, munit=munit, Tdbc=Tdbc, Ttbc=Ttbc, vrel=vrel)
    return g, got, ref


def _check(n, lattice, L, got, ref, tol, munit=2.5):
    ov = 1 << O_LAT[lattice]
    for sp in ("dm", "baryon"):
        pos, vel, ids, mass = got[sp]
        rpos, rvel, rids, rmass = ref[sp]
        assert np.array_equal(ids.astype(np.uint64), rids), sp
        rq = lattice_q(n, O_LAT[lattice], L)
        if sp == "baryon":
            rq = rq + np.asarray(O.SECOND_LATTICE_SHIFT[O_LAT[lattice]]) / n * L
        assert rel_l2(pos - rq, rpos - rq) < tol, (sp, "pos")
        assert rel_l2(vel, rvel) < tol, (sp, "vel")
        Om = COSMO_KW["Omega_b"] if sp == "baryon" else COSMO_KW["Omega_m"] - COSMO_KW["Omega_b"]
        m0 = Om * munit / (n ** 3 * ov)  # unperturbed particle mass
        if np.std(rmass) > 1e-9 * m0:  # the perturbation pmeanmass C_s delta_bc Omega_s munit
            assert rel_l2(mass - m0, rmass - m0) < tol, (sp, "mass")
        assert np.max(np.abs(mass - rmass)) <= max(tol, 1e-13) * m0, (sp, "mass")


@pytest.mark.parametrize("lattice", ["sc", "bcc", "fcc", "rsc"])
def test_two_species_eh_f64(ctx, lattice):
    """Eisenstein-Hu: delta_bc = theta_bc = 0, so uniform masses
    Omega_s munit / (n^3 overload); baryons on the secondary lattice (RSC:
    the quarter-cell shift)"""
    n, L, z = 16, 40.0, 24.0
    g, got, ref = _run(ctx, n, L, z, 2, lattice, "f64")
    _check(n, lattice, L, got, ref, 1e-12)
    ov = 1 << O_LAT[lattice]
    for sp, Om in (("dm", COSMO_KW["Omega_m"] - COSMO_KW["Omega_b"]), ("baryon", COSMO_KW["Omega_b"])):
        m = got[sp][3]
        assert np.all(m == m[0]) and m[0] == pytest.approx(Om * 2.5 / (n ** 3 * ov), rel=1e-15)
    g.close()


@pytest.mark.parametrize("lattice,order,vrel", [("sc", 3, True), ("bcc", 3, True), ("bcc", 2, False)])
def test_two_species_tables_f64(ctx, lattice, order, vrel):
    """tabulated T_delta_bc / T_theta_bc: perturbed masses and, with
    DoBaryonVrel, the species' relative-velocity term"""
    n, L, z = 32, 50.0, 24.0
    g, got, ref = _run(ctx, n, L, z, order, lattice, "f64", tables=True, vrel=vrel)
    _check(n, lattice, L, got, ref, 1e-12)
    # the masses really are perturbed, and differently per species
    assert got["dm"][3].std() > 0 and got["baryon"][3].std() > 0
    if vrel:  # the species' velocities differ by the relative-velocity term
        assert rel_l2(got["dm"][1], got["baryon"][1]) > 1e-6
    g.close()


def test_two_species_tables_f32(ctx):
    n, L, z = 32, 50.0, 24.0
    g, got, ref = _run(ctx, n, L, z, 3, "bcc", "f32", tables=True, vrel=True)
    _check(n, "bcc", L, got, ref, 1e-5)
    g.close()


def test_two_species_dm_matches_single_species(ctx):
    """with Eisenstein-Hu and no relative-velocity mode the dark matter of a
    two-species run is the single-species run, bit for bit"""
    from monofonic_gb300 import ic
    n, L, z = 32, 60.0, 30.0
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, 8)
    base = dict(ngrid=n, boxlen=L, zstart=z, lpt_order=3, lattice="bcc", precision="f32", lunit=L, vunit=L,
                pos64=False, plt=True)
    one = ic.ICGenerator(ctx, ic.ICConfig(**base), sc)
    one.set_noise(noise)
    pos1, vel1, ids1 = one.run()
    two = ic.ICGenerator(ctx, ic.ICConfig(baryons=True, munit=1.0, **base), sc)
    two.set_noise(noise)
    out = two.run_species()
    assert np.array_equal(out["dm"][0], pos1) and np.array_equal(out["dm"][1], vel1)
    assert np.array_equal(out["dm"][2], ids1)
    assert np.array_equal(out["baryon"][2], ids1 + np.uint64(2 * n ** 3))
    one.close()
    two.close()


def test_two_species_errors(ctx):
    import monofonic_gb300 as mf
    from monofonic_gb300 import ic
    n, L, z = 16, 40.0, 24.0
    cosmo, sc, _ = setup(z)
    g = ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=2, baryons=True, munit=1.0), sc)
    g.set_noise(ic.white_noise(n, 1))
    with pytest.raises(mf.MFError, match="run_species"):
        g.run()
    g.close()
    with pytest.raises(mf.MFError):  # field output needs the SC lattice
        ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=2, baryons=True, munit=1.0,
                                        out_kind="fields", lattice="bcc"), sc)
    with pytest.raises(mf.MFError):  # mass unit required
        ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=2, baryons=True, munit=0.0), sc)
    one = ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=2), sc)
    one.set_noise(ic.white_noise(n, 1))
    with pytest.raises(mf.MFError, match="one species"):
        one.run_species()
    one.close()


def _fields_run(ctx, n, L, z, order, prec, tables, vrel, munit=2.5, seed=21):
    from monofonic_gb300 import ic
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, seed)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=order, precision=prec, lunit=L, vunit=L,
                      out_kind="fields", baryons=True, baryon_vrel=vrel, munit=munit)
    Tdbc = Ttbc = tdbc = ttbc = None
    if tables:
        Tdbc, Ttbc, tdbc, ttbc = _tables(n, L)
    g = ic.ICGenerator(ctx, cfg, sc, tk_dbc=tdbc, tk_tbc=ttbc)
    g.set_noise(noise)
    got = g.run_species()
    f = O.lpt_potentials(noise, L, order, osc)
    lag = O.two_species_particles(f, L, order, osc, COSMO_KW["Omega_m"], COSMO_KW["Omega_b"], lattice=0, lunit=L,
                                  vunit=L, munit=munit, Tdbc=Tdbc, Ttbc=Ttbc, vrel=vrel)
    fb = COSMO_KW["Omega_b"] / COSMO_KW["Omega_m"]
    eul = O.eulerian_fields(f, L, order, osc, 1.0 - fb, Tdbc=Tdbc, vunit=L)
    return g, got, lag, eul


@pytest.mark.parametrize("order,tables,vrel", [(1, True, False), (2, False, False), (2, True, True), (3, True, False)])
def test_two_species_fields_f64(ctx, order, tables, vrel):
    """field output with baryons: the dark matter's Lagrangian fields and mass
    field, the baryons' semiclassical Eulerian density and velocities
    (ic_generator.cc:679-791); the Eulerian fields to rel-L2 1e-10 (phases of
    hundreds of radians)"""
    n, L, z = 32, 50.0, 24.0
    g, got, lag, eul = _fields_run(ctx, n, L, z, order, "f64", tables, vrel)
    dx, vx, _, mass = got["dm"]
    q = lattice_q(n, 0, L)
    rpos, rvel, _, rmass = lag["dm"]
    for d in range(3):
        assert rel_l2(dx[d].reshape(-1), (rpos - q)[:, d]) < 1e-12
        assert rel_l2(vx[d].reshape(-1), rvel[:, d]) < 1e-12
    m0 = (COSMO_KW["Omega_m"] - COSMO_KW["Omega_b"]) * 2.5
    rm = rmass * n ** 3  # the field is written as is, without pmeanmass
    if tables:
        assert rel_l2(mass.reshape(-1) - m0, rm - m0) < 1e-12
    assert np.max(np.abs(mass.reshape(-1) - rm)) <= 1e-13 * m0
    rho, vel = got["baryon"][0], got["baryon"][1]
    rrho, rvel_e = eul
    assert rel_l2(rho, rrho) < 1e-10
    for d in range(3):
        assert rel_l2(vel[d], rvel_e[d]) < 1e-10, d
    assert np.abs(rrho).max() > 1e-3  # a non-trivial density field
    g.close()


def test_two_species_fields_f32(ctx):
    """FP32-bulk pipeline: the Eulerian branch runs in FP64 from the FP32
    potentials; the density error follows the potentials' rounding times the
    phase (hundreds of radians), so its tolerance is 5e-3"""
    n, L, z = 32, 50.0, 24.0
    g, got, lag, eul = _fields_run(ctx, n, L, z, 3, "f32", True, True)
    q = lattice_q(n, 0, L)
    for d in range(3):
        assert rel_l2(got["dm"][0][d].reshape(-1), (lag["dm"][0] - q)[:, d]) < 1e-5
    assert rel_l2(got["baryon"][0], eul[0]) < 5e-3
    for d in range(3):
        assert rel_l2(got["baryon"][1][d], eul[1][d]) < 5e-3
    g.close()


def test_grafic2_two_species(ctx, tmp_path):
    """the GRAFIC-2 plugin with baryons: dark matter dx..vz and mass, baryon
    density and velocities; dark-matter density and baryon mass skipped"""
    from monofonic_gb300 import ic
    from monofonic_gb300.output import Grafic2Output
    from oracle import grafic2_oracle as G
    n, L, z = 32, 50.0, 24.0
    cosmo, sc, osc = setup(z)
    Om, Ob = COSMO_KW["Omega_m"], COSMO_KW["Omega_b"]
    w = Grafic2Output(ctx, str(tmp_path / "ics"), n, L, z, 100 * COSMO_KW["h"], Om, 1 - Om, Ob, baryons=True)
    assert "hydro=.true." in (tmp_path / "ics" / "ramses.nml").read_text()
    Tdbc, Ttbc, tdbc, ttbc = _tables(n, L)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=2, lunit=w.position_unit(), vunit=w.velocity_unit(),
                      out_kind="fields", baryons=True, munit=w.mass_unit())
    gen = ic.ICGenerator(ctx, cfg, sc, tk_dbc=tdbc, tk_tbc=ttbc)
    noise = ic.white_noise(n, 4)
    gen.set_noise(noise)
    w.write_ic(gen)
    gen.set_noise(noise)
    out = gen.run_species()
    hdr = G.header(n, L, z, 100 * COSMO_KW["h"], Om, 1 - Om)
    expect = {("dm", "dx"): out["dm"][0][0], ("dm", "vz"): out["dm"][1][2], ("dm", "mass"): out["dm"][3],
              ("baryon", "density"): out["baryon"][0], ("baryon", "vy"): out["baryon"][1][1]}
    for (sp, c), field in expect.items():
        assert open(G.file_name(str(tmp_path / "ics"), sp, c), "rb").read() == G.file_bytes(field, hdr), (sp, c)
    names = sorted(p.name for p in (tmp_path / "ics").iterdir())
    assert names == sorted(["ramses.nml", "ic_poscx", "ic_poscy", "ic_poscz", "ic_velcx", "ic_velcy", "ic_velcz",
                            "ic_massc", "ic_deltab", "ic_velbx", "ic_velby", "ic_velbz"])
    gen.close()
    w.close()
