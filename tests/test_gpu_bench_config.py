"""The benchmarked configuration itself (3LPT + PLT, BCC 2x512^3, L = 1000 Mpc/h,
z = 24, M = 768) in both forms on the device:

  * FP32-bulk against plain FP64, per LPT order: the growth-scaled potentials
    phi(1), phi(2), phi(3) and A(3) of both runs turned into the displacement
    field of each order (ic_generator.cc:821-858 with the Fourier gradient),
    rel-L2 <= 1e-5 each, and the particles of both runs (displacements from
    the lattice, and velocities; the FP32 positions against the FP64 ones
    rounded to float, as stored floats), rel-L2 <= 1e-5;
  * the float-pair arithmetic of the FP32 form, which carries the order sum
    and q + Psi as float pairs instead of FP64: the device helpers against
    the FP64 evaluation rounded once, on inputs shaped like this
    configuration's; the number of stored floats that differ is reported and
    must be below 1 in 10^6.

The same configuration at N = 256 is compared with the reference's own output
in tests/test_gpu_reference.py (FP64 1e-12, FP32 1e-5)."""
import numpy as np
import pytest

from tests.ic_helpers import setup

pytestmark = pytest.mark.gpu
N, L, Z, SEED = 512, 1000.0, 24.0, 20241


def _run(ctx, sc, prec, lattice="bcc", plt=True, out_kind="particles"):
    from monofonic_gb300 import ic
    cfg = ic.ICConfig(ngrid=N, boxlen=L, zstart=Z, lpt_order=3, lattice=lattice, precision=prec, plt=plt,
                      lunit=L, vunit=L, pos64=(prec == "f64"), id64=True, out_kind=out_kind)
    g = ic.ICGenerator(ctx, cfg, sc)
    g.set_noise_seed(SEED)
    pos, vel, ids = g.run()
    pots = [g.potential(w).astype(np.complex128) for w in range(6)]
    g.close()
    return pos, vel, ids, pots


def _per_order_errors(pa, pb, D):
    """rel-L2 of the displacement of each LPT order between two runs' potentials
    (unscaled; the growth factors of ic_generator.cc:550-563 applied here),
    summed over the three components, the A(3) curl term in order 3: i k_d phi_w
    (+ i k_d' A3_d'' - i k_d'' A3_d') per component, computed in k-space (equal
    to the real-space rel-L2 by Parseval), one component at a time"""
    n = N
    kf = 2 * np.pi / L
    i = np.arange(n)
    k1 = (i - (i > n // 2) * n) * kf
    k = (k1[:, None, None], k1[None, :, None], (np.arange(n // 2 + 1) * kf)[None, None, :])
    gw = [-D, -3.0 / 7.0 * D * D, D ** 3 / 3.0, D ** 3 / 7.0]
    out = {}
    for w in (1, 2, 3):
        num = den = 0.0
        for d in range(3):
            comp = []
            for pots in (pa, pb):
                t = 1j * k[d] * (pots[w - 1] * gw[w - 1])
                if w == 3:
                    dp, dpp = (d + 1) % 3, (d + 2) % 3
                    t = t + gw[3] * (1j * k[dp] * pots[3 + dpp] - 1j * k[dpp] * pots[3 + dp])
                comp.append(t)
            num += float(np.sum(np.abs(comp[0] - comp[1]) ** 2))
            den += float(np.sum(np.abs(comp[1]) ** 2))
        out[f"psi{w}"] = (num / den) ** 0.5
    return out


def test_bench_config_f32_bulk_vs_f64_per_order(ctx):
    from tests.ref_cases import lattice_q
    cosmo, sc, osc = setup(Z)
    p64, v64, i64, pot64 = _run(ctx, sc, "f64")
    p32, v32, i32, pot32 = _run(ctx, sc, "f32")
    assert np.array_equal(i32, i64)
    errs = _per_order_errors(pot32, pot64, sc.Dplus)
    del pot64, pot32
    q = lattice_q(N, "bcc", L)
    d64 = p64 - q
    # FP32 positions are stored floats (has_64bit_reals off): against the FP64
    # positions rounded to float, relative to the displacement
    errs["disp"] = float(np.linalg.norm(p32.astype(np.float64) - p64.astype(np.float32).astype(np.float64))
                         / np.linalg.norm(d64))
    errs["vel"] = float(np.linalg.norm(v32.astype(np.float64) - v64) / np.linalg.norm(v64))
    print(f"\nbench config 2x{N}^3 BCC+PLT FP32-bulk vs FP64: " + ", ".join(f"{k} {v:.3e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v < 1e-5, (k, v)


def test_float_pairs_match_fp64_rounding(ctx):
    """the float-pair helpers of the order sum (ff_axpy) and of q + Psi
    (ff_add_q) against the FP64 evaluation rounded once, on 2^28 inputs each
    shaped like the benchmarked configuration's (growth weights of z = 24,
    lattice coordinates of a 1000 Mpc/h box at N = 512)"""
    import ctypes as C
    import monofonic_gb300 as mf
    cosmo, sc, osc = setup(Z)
    ms, mq = C.c_longlong(), C.c_longlong()
    count = 1 << 28
    assert mf.lib().mf_selftest_float_pairs(ctx.ptr, count, 12345, sc.Dplus, C.byref(ms), C.byref(mq)) == 0
    print(f"\nfloat pairs vs FP64 rounded once: order sum {ms.value} of {count} differ, q+Psi {mq.value} of {count}")
    assert ms.value / count < 1e-6 and mq.value / count < 1e-6
