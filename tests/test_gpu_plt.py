"""PLT corrections (include/particle_plt.hh): the library's tables against the
oracle's restatement of init_D, and the pipeline's PLT-corrected
displacements/velocities against the oracle evaluated with the same tables."""
import numpy as np
import pytest

from oracle import lpt_oracle as O
from tests.ic_helpers import lattice_q, rel_l2, setup

pytestmark = pytest.mark.gpu


def _stable_mask(lat, ng, ref):
    """mesh points whose tables do not move under a 1e-12 perturbation of the
    dynamical matrices: where the largest eigenvalue is degenerate its
    eigenvector is not unique, and any eigensolver (GSL's included) picks an
    arbitrary one."""
    orig = np.linalg.eigh
    rng = np.random.default_rng(0)

    def pert(M):
        E = rng.standard_normal(M.shape) * 1e-12 * np.abs(M).max()
        return orig(M + (E + np.swapaxes(E, -1, -2)) / 2)

    np.linalg.eigh = pert
    try:
        alt = O.plt_tables(lat, ng)
    finally:
        np.linalg.eigh = orig
    m = np.ones(ref[0].shape, dtype=bool)
    for a, b in zip(ref, alt):
        m &= np.isclose(a, b, rtol=1e-9, atol=1e-11)
    return m


@pytest.mark.parametrize("lattice", ["sc", "bcc", "fcc"])
def test_plt_tables_match_oracle(ctx, lattice):
    from monofonic_gb300 import ic
    lat = {"sc": 0, "bcc": 1, "fcc": 2}[lattice]
    got = ic.plt_tables(ctx, lattice, 16)
    ref = O.plt_tables(lat, 16)
    stable = _stable_mask(lat, 16, ref)
    assert stable.mean() > 0.9
    for name, a, b in zip(("Dr", "Dth", "Dph", "Dvf"), got, ref):
        assert np.all(np.isfinite(a)), name
        close = np.isclose(a, b, rtol=1e-9, atol=1e-11)
        assert close[stable].mean() > 0.999, (name, close[stable].mean())


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_plt_pipeline_matches_oracle(ctx, prec, tol):
    from monofonic_gb300 import ic
    n, L, z, ng = 32, 62.5, 24.0, 16
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, 2718)
    tables = ic.plt_tables(ctx, "bcc", ng)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=3, lattice="bcc", precision=prec, plt=True,
                      plt_ngrid=ng, lunit=L, vunit=L)
    g = ic.ICGenerator(ctx, cfg, sc)
    g.set_noise(noise)
    pos, vel, ids = g.run()
    f = O.lpt_potentials(noise, L, 3, osc)
    q = lattice_q(n, 1, L)
    # oracle: set_positions / set_velocities with the PLT gradient on both sub-lattices
    rpos = np.empty((2 * n ** 3, 3))
    rvel = np.empty((2 * n ** 3, 3))
    for d in range(3):
        fr = O.c2r(O.displacement_k_plt(f, L, d, 3, tables, unit=L), n)
        rpos[:, d] = O.lattice_positions_component(fr, d, 1, L, L)
        fv = O.c2r(O.displacement_k_plt(f, L, d, 3, tables, unit=L, vel=True, vfac=osc.vfac), n)
        rvel[:, d] = O.lattice_velocities_component(fv, 1, L)
    assert rel_l2(pos - q, rpos - q) < tol
    assert rel_l2(vel, rvel) < tol
    # the correction is not a no-op
    plain = ic.ICGenerator(ctx, ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=3, lattice="bcc",
                                            precision=prec, lunit=L, vunit=L), sc)
    plain.set_noise(noise)
    ppos, pvel, _ = plain.run()
    assert rel_l2(vel, pvel) > 1e-4


@pytest.mark.parametrize("lattice", ["fcc", "rsc"])
def test_multi_shift_lattices_f64(ctx, lattice):
    """FCC and RSC read their sub-lattices through chained relative shifts,
    each preceded by the projection onto real fields (particle_generator.hh:505-522)."""
    from monofonic_gb300 import ic
    lat = {"fcc": 2, "rsc": 3}[lattice]
    n, L, z = 16, 40.0, 30.0
    cosmo, sc, osc = setup(z)
    noise = ic.white_noise(n, 31)
    cfg = ic.ICConfig(ngrid=n, boxlen=L, zstart=z, lpt_order=3, lattice=lattice, lunit=L, vunit=L)
    g = ic.ICGenerator(ctx, cfg, sc)
    g.set_noise(noise)
    pos, vel, ids = g.run()
    f = O.lpt_potentials(noise, L, 3, osc)
    rpos, rvel, rids = O.particles(f, L, 3, osc.vfac, lattice=lat, lunit=L, vunit=L)
    q = lattice_q(n, lat, L)
    assert rel_l2(pos - q, rpos - q) < 1e-12
    assert rel_l2(vel, rvel) < 1e-12
    assert np.array_equal(ids, rids)
