"""Shared set-up of the pipeline parity tests: one host cosmology feeds both
the CUDA pipeline and the oracle (scalars cross the boundary unchanged)."""
import numpy as np

from oracle import lpt_oracle as O

COSMO_KW = dict(Omega_m=0.3099, Omega_b=0.0488, h=0.6774, sigma_8=0.8102, n_s=0.9667)


def setup(zstart):
    from monofonic_gb300 import ic
    cosmo = ic.Cosmology(**COSMO_KW)
    sc = ic.cosmology_scalars(cosmo, zstart)
    p = O.cosmo_parameters(COSMO_KW["Omega_m"], COSMO_KW["Omega_b"], COSMO_KW["h"], COSMO_KW["sigma_8"],
                           COSMO_KW["n_s"])
    return cosmo, sc, O.scalars_from(p, sc.Dplus, sc.vfac, sc.pnorm)


def rel_l2(a, b):
    a = np.asarray(a)
    a = a.astype(np.complex128) if np.iscomplexobj(a) else a.astype(np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def lattice_q(n, lattice, unit=1.0):
    """unperturbed lattice positions in particle order (particle_generator.hh:524-541)."""
    idx = np.arange(n, dtype=np.float64)
    out = []
    for s in O.LATTICE_SHIFTS[lattice]:
        q = np.stack(np.meshgrid((idx + s[0]) / n, (idx + s[1]) / n, (idx + s[2]) / n, indexing="ij"), -1)
        out.append(q.reshape(-1, 3) * unit)
    return np.concatenate(out)
