"""The allocation-free convolution entry point (mf_conv_convolve2_noalloc).

It exists for callers that cannot allocate device memory -- for example a
simulation code that runs the generator in-process while its own memory pool
owns the device, or host code that must avoid the implicit synchronisation
of cudaMalloc/cudaFree.  These tests call it through the C ABI and compare it
with the allocating convolver entry point (mf_conv_convolve2) on the same
inputs and with the oracle's Orszag convolution, two calls in a row, within
the tolerances of the other convolution tests (FP64 rel-L2 1e-12, FP32 1e-5),
at the largest sizes the static scratch admits, and check that a call leaves
the device's free memory unchanged.  The file is named so that pytest runs it
last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import lpt_oracle as O

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-5}
PREC = {"f64": 0, "f32": 1}
MF_OPND_HESS, MF_OPND_SUM = 1, 2
MF_OP_ASSIGN, MF_OP_ADD = 0, 1


def _entry():
    import monofonic_gb300 as mf
    fn = mf.lib().mf_conv_convolve2_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int),
                   C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_void_p, C.c_int, C.c_double]
    return fn


def _dirs(*d):
    a = (C.c_int * 4)(*(list(d) + [0] * (4 - len(d))))
    return a


def _rel(a, b):
    return float(np.linalg.norm(a.astype(np.complex128) - b) / np.linalg.norm(b))


def _free_device_bytes():
    import torch
    free, _ = torch.cuda.mem_get_info(0)
    return free


# (precision, n): the sizes at the edge of the 48 MiB scratch (FP64 n = 96,
# 32.5 MB; FP32 n = 128, 38.3 MB), a small size for the first twiddle-table
# offsets, and n = 64 in both precisions
CASES = [("f64", 64), ("f32", 64), ("f64", 96), ("f32", 128), ("f32", 16)]


@pytest.mark.parametrize("prec,n", CASES)
def test_noalloc_matches_allocating_convolver_twice(prec, n):
    import monofonic_gb300 as mf
    fn = _entry()
    ctx = mf.Context(0)
    L = 100.0
    rng = np.random.default_rng(11 + n)
    A = O.r2c(rng.standard_normal((n, n, n)))
    B = O.r2c(rng.standard_normal((n, n, n)))
    ga, gb = mf.Grid_FFT(ctx, n, L, prec, "k"), mf.Grid_FFT(ctx, n, L, prec, "k")
    ga.set_k(A)
    gb.set_k(B)
    ref1, ref2 = mf.Grid_FFT(ctx, n, L, prec, "k"), mf.Grid_FFT(ctx, n, L, prec, "k")
    cv = mf.OrszagConvolver(ctx, n, L, prec)
    cv.convolve_Hessians(ga, (0, 1), gb, (2, 2), mf.op.assign_to(ref1))
    cv.convolve_SumOfHessians(gb, (0, 0), ga, (1, 1), (2, 2), mf.op.assign_to(ref2))
    cv.convolve_Hessians(ga, (1, 2), ga, (1, 2), mf.op.add_to(ref2))
    ctx.synchronize()
    want1, want2 = ref1.get_k(), ref2.get_k()
    # the oracle's Orszag convolution of the same (device-rounded) operands
    Ad, Bd = ga.get_k().astype(np.complex128), gb.get_k().astype(np.complex128)
    orc1 = O.orszag_conv2(O.hessian(Ad, L, 0, 1), O.hessian(Bd, L, 2, 2))
    orc2 = (O.orszag_conv2(O.hessian(Bd, L, 0, 0), O.sum_hessian(Ad, L, (1, 1), (2, 2)))
            + O.orszag_conv2(O.hessian(Ad, L, 1, 2), O.hessian(Ad, L, 1, 2)))

    out = mf.Grid_FFT(ctx, n, L, prec, "k")
    # first call: assign (the first call on a device also looks up the scratch address)
    rc = fn(ctx.stream(), n, L, PREC[prec], ga.device_ptr(), MF_OPND_HESS, _dirs(0, 1), gb.device_ptr(),
            MF_OPND_HESS, _dirs(2, 2), out.device_ptr(), MF_OP_ASSIGN, 1.0)
    assert rc == 0
    got1 = out.get_k()
    assert _rel(got1, want1) < TOL[prec]
    assert _rel(got1, orc1) < TOL[prec]
    # second call in a row, different operands, accumulated onto a prepared
    # target; it allocates no device memory
    cv.convolve_SumOfHessians(gb, (0, 0), ga, (1, 1), (2, 2), mf.op.assign_to(out))
    ctx.synchronize()
    free0 = _free_device_bytes()
    rc = fn(ctx.stream(), n, L, PREC[prec], ga.device_ptr(), MF_OPND_HESS, _dirs(1, 2), ga.device_ptr(),
            MF_OPND_HESS, _dirs(1, 2), out.device_ptr(), MF_OP_ADD, 1.0)
    assert rc == 0
    ctx.synchronize()
    assert _free_device_bytes() == free0
    got2 = out.get_k()
    assert _rel(got2, want2) < TOL[prec]
    assert _rel(got2, orc2) < TOL[prec]


def test_noalloc_rejects_sizes_beyond_its_static_scratch():
    import monofonic_gb300 as mf
    fn = _entry()
    ctx = mf.Context(0)
    g = mf.Grid_FFT(ctx, 256, 100.0, "f32", "k")
    rc = fn(ctx.stream(), 256, 100.0, 1, g.device_ptr(), MF_OPND_HESS, _dirs(0, 0), g.device_ptr(), MF_OPND_HESS,
            _dirs(1, 1), g.device_ptr(), MF_OP_ASSIGN, 1.0)
    assert rc == 2  # MF_ERR_SHAPE
    rc = fn(ctx.stream(), 128, 100.0, 0, g.device_ptr(), MF_OPND_HESS, _dirs(0, 0), g.device_ptr(), MF_OPND_HESS,
            _dirs(1, 1), g.device_ptr(), MF_OP_ASSIGN, 1.0)
    assert rc == 2  # FP64 at n = 128 needs 77 MB > 48 MiB
