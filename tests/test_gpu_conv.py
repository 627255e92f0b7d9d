"""Orszag 3/2 and aliased convolutions (include/convolution.hh:296-669) and
output operators (include/operators.hh:25-35) against the oracle."""
import numpy as np
import pytest

from oracle import lpt_oracle as O

pytestmark = pytest.mark.gpu
TOL = {"f64": 1e-12, "f32": 1e-5}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def field_k(n, seed):
    rng = np.random.default_rng(seed)
    return O.r2c(rng.standard_normal((n, n, n)))


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("n", [16, 32, 64])
def test_hessians2_assign(ctx, n, prec):
    import monofonic_gb300 as mf
    L = 100.0
    A, B = field_k(n, 1), field_k(n, 2)
    ga, gb, out = (mf.Grid_FFT(ctx, n, L, prec, "k") for _ in range(3))
    ga.set_k(A); gb.set_k(B)
    cv = mf.OrszagConvolver(ctx, n, L, prec)
    cv.convolve_Hessians(ga, (0, 1), gb, (2, 2), mf.op.assign_to(out))
    ref = O.orszag_conv2(O.hessian(A, L, 0, 1), O.hessian(B, L, 2, 2))
    assert rel_l2(out.get_k(), ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ops_chain_and_invlap(ctx, prec):
    """phi(2) source sum as in src/ic_generator.cc:471-488, fused inverse Laplacian."""
    import monofonic_gb300 as mf
    n, L = 32, 200.0
    P = field_k(n, 3)
    phi, out = mf.Grid_FFT(ctx, n, L, prec, "k"), mf.Grid_FFT(ctx, n, L, prec, "k")
    phi.set_k(P)
    cv = mf.OrszagConvolver(ctx, n, L, prec)
    cv.convolve_SumOfHessians(phi, (0, 0), phi, (1, 1), (2, 2), mf.op.assign_to(out))
    cv.convolve_Hessians(phi, (1, 1), phi, (2, 2), mf.op.add_to(out))
    cv.convolve_Hessians(phi, (0, 1), phi, (0, 1), mf.op.subtract_from(out))
    cv.convolve_Hessians(phi, (0, 2), phi, (0, 2), mf.op.multiply_add_to(out, -1.0))
    cv.convolve_Hessians(phi, (1, 2), phi, (1, 2), mf.op.subtract_from(out), invlap=True)
    H = lambda a, b: O.hessian(P, L, a, b)
    s = O.orszag_conv2(H(0, 0), O.sum_hessian(P, L, (1, 1), (2, 2)))
    s = s + O.orszag_conv2(H(1, 1), H(2, 2))
    s = s - O.orszag_conv2(H(0, 1), H(0, 1))
    s = s - O.orszag_conv2(H(0, 2), H(0, 2))
    s = s - O.orszag_conv2(H(1, 2), H(1, 2))
    ref = O.inverse_laplacian(s, L)
    assert rel_l2(out.get_k(), ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_convolve3_two_stage(ctx, prec):
    """convolve3 = two chained convolve2 with the intermediate truncated and
    Nyquist-zeroed (convolution.hh:543-549)."""
    import monofonic_gb300 as mf
    n, L = 32, 100.0
    P = field_k(n, 4)
    phi, out = mf.Grid_FFT(ctx, n, L, prec, "k"), mf.Grid_FFT(ctx, n, L, prec, "k")
    phi.set_k(P)
    cv = mf.OrszagConvolver(ctx, n, L, prec)
    cv.convolve_Hessians(phi, (0, 0), phi, (1, 1), phi, (2, 2), mf.op.assign_to(out))
    ref = O.orszag_conv3(O.hessian(P, L, 0, 0), O.hessian(P, L, 1, 1), O.hessian(P, L, 2, 2))
    assert rel_l2(out.get_k(), ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_difference_and_gradients(ctx, prec):
    import monofonic_gb300 as mf
    n, L = 16, 64.0
    A, B = field_k(n, 5), field_k(n, 6)
    ga, gb, out = (mf.Grid_FFT(ctx, n, L, prec, "k") for _ in range(3))
    ga.set_k(A); gb.set_k(B)
    cv = mf.OrszagConvolver(ctx, n, L, prec)
    cv.convolve_DifferenceOfHessians(ga, (1, 2), gb, (1, 1), (2, 2), mf.op.assign_to(out))
    ref = O.orszag_conv2(O.hessian(A, L, 1, 2), O.sum_hessian(B, L, (1, 1), (2, 2), sign=-1))
    assert rel_l2(out.get_k(), ref) < TOL[prec]
    cv.convolve_Gradients(ga, (0,), gb, (2,), mf.op.assign_to(out))
    g = O.ggrids(n, L)
    ref = O.orszag_conv2((1j * g[0]) * A, (1j * g[2]) * B)
    assert rel_l2(out.get_k(), ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_naive_convolver(ctx, prec):
    import monofonic_gb300 as mf
    n, L = 32, 100.0
    A, B, Cc = field_k(n, 7), field_k(n, 8), field_k(n, 9)
    ga, gb, gc, out = (mf.Grid_FFT(ctx, n, L, prec, "k") for _ in range(4))
    ga.set_k(A); gb.set_k(B); gc.set_k(Cc)
    cv = mf.NaiveConvolver(ctx, n, L, prec)
    cv.convolve_Hessians(ga, (0, 0), gb, (1, 2), mf.op.assign_to(out))
    ref = O.naive_conv2(O.hessian(A, L, 0, 0), O.hessian(B, L, 1, 2))
    assert rel_l2(out.get_k(), ref) < TOL[prec]
    cv.convolve_Hessians(ga, (0, 0), gb, (1, 1), gc, (2, 2), mf.op.assign_to(out))
    ref = O.naive_conv3(O.hessian(A, L, 0, 0), O.hessian(B, L, 1, 1), O.hessian(Cc, L, 2, 2))
    assert rel_l2(out.get_k(), ref) < TOL[prec]
