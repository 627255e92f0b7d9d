"""Failure handling on the device without a fault: the bounded mbarrier wait
that guards every TMA-pipelined kernel (monofonic_gb300/csrc/mf_tma.cuh) runs
out on a barrier nothing arrives on, the kernel returns, the call reports
MF_ERR_TIMEOUT (the reference has no device path; its failures are
exceptions, src/main.cc:242-252), and the context keeps working."""
import numpy as np
import pytest

from oracle import lpt_oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives():
    import monofonic_gb300 as mf
    from monofonic_gb300._lib import MF_ERR_TIMEOUT, MF_ERR_ARG
    ctx = mf.Context(0)
    lib = mf.lib()
    assert lib.mf_selftest_bounded_wait(ctx.ptr, 1 << 12) == MF_ERR_TIMEOUT
    assert b"bounded device wait" in lib.mf_last_error(ctx.ptr)
    # the flag was cleared: a second run times out again on its own, and an
    # out-of-range budget is refused before any launch
    assert lib.mf_selftest_bounded_wait(ctx.ptr, 1 << 10) == MF_ERR_TIMEOUT
    assert lib.mf_selftest_bounded_wait(ctx.ptr, 0) == MF_ERR_ARG
    ctx.synchronize()
    # the context still computes correctly after the timeouts
    n = 32
    x = np.random.default_rng(5).standard_normal((n, n, n))
    g = mf.Grid_FFT(ctx, n, 100.0, "f64")
    g.set_real(x)
    g.FourierTransformForward()
    X = g.get_k()
    ref = O.r2c(x)
    assert np.linalg.norm(X - ref) / np.linalg.norm(ref) < 1e-13
