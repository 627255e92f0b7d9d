"""3LPT at N=256 (Orszag M=384), SC lattice, box 500 Mpc/h, z_start=24,
Eisenstein-Hu, seeded N(0,1) noise: the plain FP64 form and the FP32-bulk form
against the FP64 oracle, per LPT order (psi1, psi2, psi3 including the A3
transverse term) and for the velocities.  Tolerances: FP64 rel-L2 <= 1e-12,
FP32-bulk rel-L2 <= 1e-5.  The errors are printed (pytest -s) for the record."""
import os

import numpy as np
import pytest

from oracle import lpt_oracle as O
from tests.ic_helpers import rel_l2, setup

pytestmark = pytest.mark.gpu
N, L, Z, SEED = 256, 500.0, 24.0, 12345
TOL = {"f64": 1e-12, "f32": 1e-5}


@pytest.fixture(scope="module")
def reference():
    from monofonic_gb300 import ic
    O.set_fft_workers(os.cpu_count() or 1)
    cosmo, sc, osc = setup(Z)
    noise = ic.white_noise(N, SEED)
    f = O.lpt_potentials(noise, L, 3, osc)
    return sc, osc, noise, f


def _order_only(f, w):
    z = np.zeros_like(f.phi)
    return O.LPTFields(phi=f.phi if w == 1 else z, phi2=f.phi2 if w == 2 else z, phi3=f.phi3 if w == 3 else z,
                       A3=f.A3 if w == 3 else [z, z, z])


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_config2_per_order_errors(ctx, reference, prec):
    from monofonic_gb300 import ic
    sc, osc, noise, f = reference
    cfg = ic.ICConfig(ngrid=N, boxlen=L, zstart=Z, lpt_order=3, precision=prec, out_kind="fields")
    g = ic.ICGenerator(ctx, cfg, sc)
    g.set_noise(noise)
    dx, vx, _ = g.run()
    D = sc.Dplus
    gw = [-D, -3.0 / 7.0 * D * D, D ** 3 / 3.0, D ** 3 / 7.0]
    pot = [g.potential(w).astype(np.complex128) for w in range(6)]
    fg = O.LPTFields(phi=pot[0] * gw[0], phi2=pot[1] * gw[1], phi3=pot[2] * gw[2], A3=[p * gw[3] for p in pot[3:6]])
    g.close()
    errs = {}
    for w in (1, 2, 3):
        a, b = _order_only(fg, w), _order_only(f, w)
        num = den = 0.0
        for d in range(3):
            pa = O.c2r(O.displacement_k(a, L, d, 3), N)
            pb = O.c2r(O.displacement_k(b, L, d, 3), N)
            num += float(np.sum((pa - pb) ** 2))
            den += float(np.sum(pb ** 2))
        errs[f"psi{w}"] = (num / den) ** 0.5
    num = den = numv = denv = 0.0
    for d in range(3):
        rd = O.c2r(O.displacement_k(f, L, d, 3), N)
        rv = O.c2r(O.displacement_k(f, L, d, 3, vel=True, vfac=osc.vfac), N)
        num += float(np.sum((dx[d] - rd) ** 2)); den += float(np.sum(rd ** 2))
        numv += float(np.sum((vx[d] - rv) ** 2)); denv += float(np.sum(rv ** 2))
    errs["psi_total"] = (num / den) ** 0.5
    errs["v"] = (numv / denv) ** 0.5
    print(f"\nconfig2 N={N} {prec}: " + ", ".join(f"{k} {v:.3e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v < TOL[prec], (k, v)
