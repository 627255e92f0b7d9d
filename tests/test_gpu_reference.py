"""The CUDA pipeline against the reference itself: every fixture in
tests/golden/ref_*.npz is what oracle/_ref -- the reference's unmodified
sources compiled against the project shims -- handed its output plugin for
one configuration (tests/ref_cases.py).  The pipeline runs the same
configuration through the C ABI with the device white-noise generator (the
project RNG plugin's bits) and the scalars the reference computed.

Tolerances: FP64 rel-L2 1e-12 on displacements (positions minus the
lattice), velocities, masses and fields, IDs exact; FP32-bulk 1e-5.  Large
cases are compared on the fixture's fixed sample of particles / cells and on
the sum of squares over all of them."""
import numpy as np
import pytest

from tests import ref_cases as R

pytestmark = pytest.mark.gpu

ALL = list(R.CASES)
F64_TOL, F32_TOL = 1e-12, 1e-5


def _spt_density(phi_k, n, L, Dplus):
    """the reference's field-output density, -k^2 phi with phi scaled by
    g1 = -D+ (ic_generator.cc:556, 934-941), from the pipeline's unscaled phi"""
    from oracle import lpt_oracle as O
    kx, ky, kz = O.kgrids(n, L)
    return O.c2r(Dplus * (kx * kx + ky * ky + kz * kz) * phi_k.astype(np.complex128), n)


@pytest.mark.parametrize("name", ALL)
def test_pipeline_f64_matches_reference(ctx, name):
    case, scalars, want = R.load_fixture(name)
    out = R.gpu_outputs(ctx, case, scalars, "f64")
    got = R.to_fixture_keys(case, out)
    if "_phi_k" in out and ("dm_density" in want or "dm_density@idx" in want):
        got["dm_density"] = _spt_density(out["_phi_k"], case["ngrid"], case["boxlen"], scalars["Dplus"])
    want = {k: v for k, v in want.items() if not k.endswith("_pk")}
    R.compare(got, want, F64_TOL, name)


@pytest.mark.parametrize("name", ["lpt3_bcc_n16", "lpt3_bcc_plt_n16", "lpt3_fcc_n16", "config1_lpt2_sc_n64_fields",
                                  "config2_lpt3_sc_n256", "config3_lpt3_bcc_plt_n256"])
def test_pipeline_f32_bulk_matches_reference(ctx, name):
    """the FP32-bulk form against the reference's FP64 output"""
    case, scalars, want = R.load_fixture(name)
    got = R.to_fixture_keys(case, R.gpu_outputs(ctx, case, scalars, "f32"))
    want = {k: v for k, v in want.items() if not k.endswith("_pk") and not k.startswith("dm_density")}
    R.compare(got, want, F32_TOL, name)


@pytest.mark.parametrize("name", ["config1_lpt2_sc_n64_fields", "fields_baryons_eulerian_lpt2_sc_n16"])
def test_power_spectrum_of_the_ic_matches_reference(ctx, name):
    """Compute_PowerSpectrum (src/grid_fft.cc:1133-1210) of the IC's density,
    on the device (mf_grid_power_spectrum) for the pipeline's own field,
    against the reference's estimator on the reference's field (full
    precision): bins, mode counts exact, P and its error to 1e-12"""
    import monofonic_gb300 as mf
    case, scalars, want = R.load_fixture(name)
    out = R.gpu_outputs(ctx, case, scalars, "f64")
    n, L = case["ngrid"], case["boxlen"]
    dens = _spt_density(out["_phi_k"], n, L, scalars["Dplus"])
    g = mf.Grid_FFT(ctx, n, L, "f64")
    g.set_real(dens)
    k, P, eP, cnt = g.Compute_PowerSpectrum()
    pk = want["dm_pk"]
    m = pk[:, 3] > 0
    assert np.array_equal(cnt[m], pk[m, 3].astype(np.int64))
    for a, b in ((k[m], pk[m, 0]), (P[m], pk[m, 1]), (eP[m], pk[m, 2])):
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-12
