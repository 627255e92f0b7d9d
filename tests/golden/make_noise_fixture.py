"""Writes tests/golden/noise_n16_seed12345.npy: the project RNG plugin's white
noise (mf_white_noise_host, n = 16, seed 12345) as float64.  The fixture pins
the generator's bits across machines: the host plugin on any architecture and
the device generator must reproduce it exactly."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from monofonic_gb300 import ic  # noqa: E402


def main():
    a = ic.white_noise(16, 12345, nthreads=1)
    np.save(os.path.join(HERE, "noise_n16_seed12345.npy"), a)
    print("wrote", a.shape, a.dtype, float(a.std()))


if __name__ == "__main__":
    main()
