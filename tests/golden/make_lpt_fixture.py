"""Writes tests/golden/lpt3_bcc_n16_seed777.npz: the oracle's 3LPT particles
on a BCC lattice (2 x 16^3, L = 31.25 Mpc/h, z = 24, FP64) for the project
RNG plugin's noise (seed 777) and the host cosmology scalars of the default
parameter set.  The fixture pins the oracle itself (tests/test_cpu_oracle.py
re-derives it) and gives the GPU pipeline a committed target
(tests/test_gpu_ic.py)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import lpt_oracle as O  # noqa: E402
from tests.ic_helpers import setup  # noqa: E402
from monofonic_gb300 import ic  # noqa: E402

N, L, Z, ORDER, LATTICE, SEED = 16, 500.0 * 16 / 256, 24.0, 3, 1, 777


def fixture():
    _, sc, osc = setup(Z)
    noise = ic.white_noise(N, SEED)
    f = O.lpt_potentials(noise, L, ORDER, osc)
    pos, vel, ids = O.particles(f, L, ORDER, osc.vfac, lattice=LATTICE, lunit=L, vunit=L)
    return dict(pos=pos, vel=vel, ids=ids, n=N, boxlen=L, zstart=Z, order=ORDER, lattice=LATTICE, seed=SEED,
                Dplus=sc.Dplus, vfac=sc.vfac, pnorm=sc.pnorm)


def main():
    d = fixture()
    path = os.path.join(HERE, "lpt3_bcc_n16_seed777.npz")
    np.savez_compressed(path, **d)
    print("wrote", path, d["pos"].shape, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
