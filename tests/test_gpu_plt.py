"""PLT corrections (include/particle_plt.hh): the library's tables against the
oracle's restatement of init_D, and the pipeline's PLT-corrected
displacements/velocities against the oracle evaluated with the same tables."""
import numpy as np
import pytest

from oracle import lpt_oracle as O
from tests.ic_helpers import lattice_q, rel_l2, setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lattice", ["sc", "bcc"])
def test_plt_tables_match_oracle(ctx, lattice):
    from monofonic_gb300 import ic
    lat = {"sc": 0, "bcc": 1}[lattice]
    got = ic.plt_tables(ctx, lattice, 16)
    ref = O.plt_tables(lat, 16)
    for name, a, b in zip(("Dr", "Dth", "Dph", "Dvf"), got, ref):
        assert np.all(np.isfinite(a)), name
        # eigenvectors of a degenerate largest eigenvalue are not unique; all
        # other mesh points agree to rounding
        close = np.isclose(a, b, rtol=1e-9, atol=1e-11)
        assert close.mean() > 0.99, (name, close.mean())


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
