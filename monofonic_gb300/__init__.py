"""monofonic_gb300: GB300 (sm_103a) nLPT field pipeline of monofonIC.

Python mirror of the reference's field/convolver/operator API over the C ABI
of libmfgpu (include/monofonic_gb300.h):

    Grid_FFT            include/grid_fft.hh:40-914
    OrszagConvolver     include/convolution.hh:429-669
    NaiveConvolver      include/convolution.hh:296-426
    op.assign_to ...    include/operators.hh:25-35

All arithmetic runs in CUDA kernels; the Python layer only moves handles.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import MFError

__all__ = ["Context", "Grid_FFT", "OrszagConvolver", "NaiveConvolver", "op", "MFError", "lib", "grid_sizes",
           "grid_wave_vector", "grid_gradient", "grid_laplacian"]


def lib():
    return L.load()


def _check(ctx_ptr, rc):
    if rc != L.MF_OK:
        msg = lib().mf_last_error(ctx_ptr)
        raise MFError(rc, msg.decode() if msg else "")


_PREC = {"f64": L.MF_PREC_F64, "f32": L.MF_PREC_F32, "double": L.MF_PREC_F64, "float": L.MF_PREC_F32}


class Context:
    """A device context: one CUDA stream, twiddle tables, error state."""

    def __init__(self, device: int = 0):
        p = C.c_void_p()
        rc = lib().mf_ctx_create(device, C.byref(p))
        if rc != L.MF_OK:
            raise MFError(rc, f"mf_ctx_create(device={device}) failed")
        self.ptr = p

    KERNEL_KINDS = ("conv_xinv", "conv_yinv", "conv_z", "conv_yfwd", "conv_xfwd", "fft_z", "fft_col", "pointwise")

    def synchronize(self):
        _check(self.ptr, lib().mf_ctx_synchronize(self.ptr))

    def stream(self) -> int:
        """cudaStream_t of the context (an integer handle)."""
        s = C.c_void_p()
        _check(self.ptr, lib().mf_ctx_stream(self.ptr, C.byref(s)))
        return s.value or 0

    def launch_counts(self) -> dict:
        a = np.zeros(8, dtype=np.int64)
        _check(self.ptr, lib().mf_ctx_launch_counts(self.ptr, a.ctypes.data, 8))
        return dict(zip(self.KERNEL_KINDS, a.tolist()))

    def fma_rate(self, prec: str = "f64") -> float:
        """measured FMA throughput in TFLOP/s"""
        r = C.c_double()
        _check(self.ptr, lib().mf_probe_fma_rate(self.ptr, _PREC[prec], C.byref(r)))
        return r.value

    def profile(self, enable: bool):
        _check(self.ptr, lib().mf_ctx_profile(self.ptr, int(enable)))

    def profile_read(self) -> dict:
        """{kind: (device ms summed over launches, launches)} since the last read."""
        ms = np.zeros(8)
        cnt = np.zeros(8, dtype=np.int64)
        _check(self.ptr, lib().mf_ctx_profile_read(self.ptr, ms.ctypes.data, cnt.ctypes.data, 8))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_KINDS)}

    def close(self):
        """Destroy the context; refused (kept alive) while grids,
        convolvers or pipelines created on it still exist."""
        if getattr(self, "ptr", None):
            if lib().mf_ctx_destroy(self.ptr) == L.MF_OK:
                self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def grid_sizes(n: int, space: str):
    """Grid_FFT::size(0..3) (src/grid_fft.cc:100-110, single process): the
    three extents and the stored row length, (n, n, n, n+2) in real space and
    (n, n, n/2+1, n/2+1) in k-space"""
    return (n, n, n, n + 2) if space == "r" else (n, n, n // 2 + 1, n // 2 + 1)


def grid_wave_vector(n: int, boxlen: float, i: int, j: int, k: int, dtype=np.float64) -> np.ndarray:
    """Grid_FFT::get_k (include/grid_fft.hh:281-296, single process): per axis
    (idx - n*[idx > n/2]) * 2pi/L in the grid's real type, the Nyquist index
    staying positive"""
    kfac = dtype(2.0 * np.pi / boxlen)
    half = n // 2
    return np.array([(dtype(x) - dtype(x > half) * dtype(n)) * kfac for x in (i, j, k)], dtype=dtype)


def grid_gradient(n: int, boxlen: float, idim: int, ijk, dtype=np.float64) -> complex:
    """Grid_FFT::gradient (include/grid_fft.hh:376-385): i k_idim, zero at the
    Nyquist index of that axis"""
    x = int(ijk[idim])
    if x == n // 2:
        return complex(0.0, 0.0)
    return complex(0.0, float(grid_wave_vector(n, boxlen, *ijk, dtype=dtype)[idim]))


def grid_laplacian(n: int, boxlen: float, ijk, dtype=np.float64) -> float:
    """Grid_FFT::laplacian (include/grid_fft.hh:387-390): -|k|^2"""
    kv = grid_wave_vector(n, boxlen, *ijk, dtype=dtype)
    return float(-(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]))


class Grid_FFT:
    """Device-resident Grid_FFT<real_t>: n^3 real grid in the padded in-place
    layout (n+2)*n*n reals, k-space (n, n, n/2+1) complex in place."""

    def __init__(self, ctx: Context, n: int, boxlen: float, prec: str = "f64", space: str = "r"):
        self.ctx, self.n, self.L = ctx, int(n), float(boxlen)
        self.prec = prec
        self.dtype = np.float64 if _PREC[prec] == L.MF_PREC_F64 else np.float32
        self.cdtype = np.complex128 if self.dtype == np.float64 else np.complex64
        p = C.c_void_p()
        sp = L.MF_SPACE_K if space == "k" else L.MF_SPACE_R
        _check(ctx.ptr, lib().mf_grid_create(ctx.ptr, self.n, self.L, _PREC[prec], sp, C.byref(p)))
        self.ptr = p

    # -- state ------------------------------------------------------------
    @property
    def space(self):
        s = C.c_int()
        lib().mf_grid_info(self.ptr, None, None, C.byref(s), None, None)
        return "k" if s.value == L.MF_SPACE_K else "r"

    def device_ptr(self):
        d = C.c_void_p()
        lib().mf_grid_info(self.ptr, None, None, None, C.byref(d), None)
        return d.value

    # -- host transfer ------------------------------------------------------
    def upload_padded(self, arr: np.ndarray, space: str):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        assert a.size == (self.n + 2) * self.n * self.n
        _check(self.ctx.ptr, lib().mf_grid_upload(self.ptr, a.ctypes.data, L.MF_SPACE_K if space == "k" else L.MF_SPACE_R))

    def download_padded(self) -> np.ndarray:
        a = np.empty((self.n, self.n, self.n + 2), dtype=self.dtype)
        _check(self.ctx.ptr, lib().mf_grid_download(self.ptr, a.ctypes.data))
        return a

    def set_real(self, x: np.ndarray):
        """relem assignment of an (n,n,n) array (host upload)."""
        a = np.zeros((self.n, self.n, self.n + 2), dtype=self.dtype)
        a[:, :, : self.n] = x
        self.upload_padded(a, "r")

    def fill_real64(self, x: np.ndarray):
        """RNG_plugin::Fill_Grid equivalent: upload an (n,n,n) float64 field."""
        a = np.ascontiguousarray(x, dtype=np.float64)
        assert a.shape == (self.n,) * 3
        _check(self.ctx.ptr, lib().mf_grid_fill_real64(self.ptr, a.ctypes.data))

    def set_k(self, X: np.ndarray):
        """kelem assignment of an (n,n,n/2+1) complex array (host upload)."""
        a = np.ascontiguousarray(X, dtype=self.cdtype)
        self.upload_padded(a.view(self.dtype).reshape(self.n, self.n, self.n + 2), "k")

    def get_real(self) -> np.ndarray:
        return self.download_padded()[:, :, : self.n].copy()

    def get_k(self, i=None, j=None, k=None) -> np.ndarray:
        """with indices: the wave vector of mode (i, j, k), Grid_FFT::get_k
        (include/grid_fft.hh:281-296); without: the k-space field as an
        (n, n, n/2+1) complex host array"""
        if i is not None:
            if j is None or k is None:
                raise TypeError("get_k takes three mode indices (i, j, k) or none")
            return grid_wave_vector(self.n, self.L, i, j, k, self.dtype)
        return self.download_padded().view(self.cdtype).reshape(self.n, self.n, self.n // 2 + 1).copy()

    # -- element reads (include/grid_fft.hh:179-211) ------------------------
    def _read(self, idx: int, count: int, dtype) -> np.ndarray:
        if not 0 <= idx < count:
            raise IndexError(f"element {idx} outside the grid's {count} stored elements")
        self.ctx.synchronize()  # the grid's kernels run on the context's stream
        out = np.empty(1, dtype=dtype)
        rc = lib().mf_copy_to_host(out.ctypes.data, C.c_void_p(self.device_ptr() + idx * out.itemsize),
                                   out.itemsize)
        if rc != L.MF_OK:
            raise MFError(rc, "mf_copy_to_host")
        return out

    def relem(self, i: int, j: int = None, k: int = None):
        """relem(i, j, k) or relem(idx): one real element of the stored
        (n, n, n+2) layout, read from the device"""
        idx = i if j is None else (i * self.n + j) * (self.n + 2) + k
        return self._read(idx, (self.n + 2) * self.n * self.n, self.dtype)[0]

    def kelem(self, i: int, j: int = None, k: int = None):
        """kelem(i, j, k) or kelem(idx): one complex mode of the stored
        (n, n, n/2+1) layout, read from the device"""
        idx = i if j is None else (i * self.n + j) * (self.n // 2 + 1) + k
        return self._read(idx, self.n * self.n * (self.n // 2 + 1), self.cdtype)[0]

    def get_r(self, i: int, j: int, k: int) -> np.ndarray:
        """Grid_FFT::get_r (include/grid_fft.hh:218-228): cell position (i, j, k) * dx"""
        dx = self.dtype(self.L / self.n)
        return np.array([self.dtype(i) * dx, self.dtype(j) * dx, self.dtype(k) * dx], dtype=self.dtype)

    def reset(self):
        """Grid_FFT::reset: free the device memory (the object is unusable after)"""
        self.close()

    # -- functions of the field on the host mirror (grid_fft.hh:450-810) ----
    # The reference loops a functor over every element on the CPU.  Here the
    # field is read back, f is applied to whole numpy arrays (broadcasting
    # replaces the element loop) and the result is written back, in the
    # space the grid is in.  The pipeline's own k-space operators run as
    # CUDA kernels; these are for arbitrary user functions.
    def _k_arrays(self):
        n = self.n
        kfac = self.dtype(2.0 * np.pi / self.L)
        idx = np.arange(n)
        k1 = ((idx.astype(self.dtype) - (idx > n // 2).astype(self.dtype) * self.dtype(n)) * kfac).astype(self.dtype)
        return k1[:, None, None], k1[None, :, None], k1[None, None, : n // 2 + 1]

    def _r_arrays(self):
        dx = self.dtype(self.L / self.n)
        r1 = (np.arange(self.n).astype(self.dtype) * dx).astype(self.dtype)
        return r1[:, None, None], r1[None, :, None], r1[None, None, :]

    def _put_k(self, X):
        a = np.ascontiguousarray(np.broadcast_to(X, (self.n, self.n, self.n // 2 + 1)), dtype=self.cdtype)
        self.upload_padded(a.view(self.dtype).reshape(self.n, self.n, self.n + 2), self.space)

    def _put_r(self, x):
        a = self.download_padded()
        a[:, :, : self.n] = x
        self.upload_padded(a, self.space)

    def apply_function_k(self, f):
        """kelem <- f(kelem) (grid_fft.hh:450-465)"""
        self._put_k(f(self.get_k()))

    def apply_function_r(self, f):
        """relem <- f(relem) (grid_fft.hh:467-482)"""
        self._put_r(f(self.get_real()))

    def apply_function_k_dep(self, f):
        """kelem <- f(kelem, k) with k = (kx, ky, kz) broadcastable arrays
        (grid_fft.hh:776-791)"""
        self._put_k(f(self.get_k(), self._k_arrays()))

    def apply_function_r_dep(self, f):
        """relem <- f(relem, r) with r = (x, y, z) cell positions
        (grid_fft.hh:793-808)"""
        self._put_r(f(self.get_real(), self._r_arrays()))

    def assign_function_of_grids_r(self, f, *grids):
        """relem <- f(g1.relem, g2.relem, ...) (grid_fft.hh:697-714)"""
        self._put_r(f(*[g.get_real() for g in grids]))

    def assign_function_of_grids_k(self, f, *grids):
        """kelem <- f(g1.kelem, g2.kelem, ...) (grid_fft.hh:716-734)"""
        self._put_k(f(*[g.get_k() for g in grids]))

    def assign_function_of_grids_ijk(self, f, *grids):
        """kelem <- f((i, j, k), g1.kelem, ...) with broadcastable index arrays
        (grid_fft.hh:736-754)"""
        n = self.n
        ijk = (np.arange(n)[:, None, None], np.arange(n)[None, :, None], np.arange(n // 2 + 1)[None, None, :])
        self._put_k(f(ijk, *[g.get_k() for g in grids]))

    def assign_function_of_grids_kdep(self, f, *grids):
        """kelem <- f(k, g1.kelem, ...) (grid_fft.hh:756-774)"""
        self._put_k(f(self._k_arrays(), *[g.get_k() for g in grids]))

    # -- index helpers (host arithmetic, include/grid_fft.hh:121-390) -------
    def size(self, i: int) -> int:
        return grid_sizes(self.n, self.space)[i]

    def get_idx(self, i: int, j: int, k: int) -> int:
        """linear index of element (i, j, k) in the stored layout"""
        sz = grid_sizes(self.n, self.space)
        return (i * sz[1] + j) * sz[3] + k

    def get_dx(self, idim: int = 0) -> float:
        return float(self.dtype(self.L / self.n))

    def get_k3(self, i: int, j: int, k: int):
        return (i, j, k)

    def gradient(self, idim: int, ijk) -> complex:
        return grid_gradient(self.n, self.L, idim, ijk, self.dtype)

    def laplacian(self, ijk) -> float:
        return grid_laplacian(self.n, self.L, ijk, self.dtype)

    # -- Grid_FFT methods ---------------------------------------------------
    def fill_white_noise(self, seed: int):
        """RNG_plugin::Fill_Grid (random_plugin.hh:37): the project plugin's
        N(0,1) field generated on the device (bit-identical to the host plugin)"""
        _check(self.ctx.ptr, lib().mf_grid_fill_white_noise(self.ptr, C.c_uint64(int(seed))))

    def FourierTransformForward(self, do_transform: bool = True):
        _check(self.ctx.ptr, lib().mf_grid_fft_forward(self.ptr, int(do_transform)))

    def FourierTransformBackward(self, do_transform: bool = True):
        _check(self.ctx.ptr, lib().mf_grid_fft_backward(self.ptr, int(do_transform)))

    def zero(self):
        _check(self.ctx.ptr, lib().mf_grid_zero(self.ptr))

    def __imul__(self, x: float):
        _check(self.ctx.ptr, lib().mf_grid_scale(self.ptr, float(x)))
        return self

    def zero_DC_mode(self):
        _check(self.ctx.ptr, lib().mf_grid_zero_dc(self.ptr))

    def apply_InverseLaplacian(self):
        _check(self.ctx.ptr, lib().mf_grid_inverse_laplacian(self.ptr))

    def shift_field(self, s, transform_back: bool = True):
        arr = (C.c_double * 3)(*[float(v) for v in s])
        _check(self.ctx.ptr, lib().mf_grid_shift(self.ptr, arr, int(transform_back)))

    def Compute_PowerSpectrum(self):
        cap = self.n
        k, P, eP = (np.zeros(cap) for _ in range(3))
        cnt = np.zeros(cap, dtype=np.int64)
        nb = C.c_int()
        _check(self.ctx.ptr, lib().mf_grid_power_spectrum(self.ptr, k.ctypes.data, P.ctypes.data, eP.ctypes.data,
                                                          cnt.ctypes.data, cap, C.byref(nb)))
        m = nb.value
        return k[:m], P[:m], eP[:m], cnt[:m]

    def Write_PowerSpectrum(self, ofname: str):
        """Write_PowerSpectrum (grid_fft.cc:1104-1131): the binned P(k) as text"""
        _check(self.ctx.ptr, lib().mf_grid_write_power_spectrum(self.ptr, ofname.encode()))

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_grid_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Op:
    """Output operator descriptor (include/operators.hh:25-35)."""

    def __init__(self, grid, kind, x=1.0):
        self.grid, self.kind, self.x = grid, kind, x


class op:
    @staticmethod
    def assign_to(g):
        return _Op(g, L.MF_OP_ASSIGN)

    @staticmethod
    def add_to(g):
        return _Op(g, L.MF_OP_ADD)

    @staticmethod
    def subtract_from(g):
        return _Op(g, L.MF_OP_SUB)

    @staticmethod
    def multiply_add_to(g, x):
        return _Op(g, L.MF_OP_AXPY, float(x))


def _opnd(g, kind, d=()):
    o = L.mf_operand()
    o.grid = g.ptr
    o.kind = kind
    for i, v in enumerate(d):
        o.d[i] = int(v)
    return o


class _Convolver:
    KIND = L.MF_CONV_ORSZAG

    def __init__(self, ctx: Context, n: int, boxlen: float, prec: str = "f64"):
        self.ctx = ctx
        p = C.c_void_p()
        _check(ctx.ptr, lib().mf_conv_create(ctx.ptr, int(n), float(boxlen), _PREC[prec], self.KIND, C.byref(p)))
        self.ptr = p

    def _c2(self, a, b, o: _Op, invlap=False):
        fn = lib().mf_conv_convolve2_invlap if invlap else lib().mf_conv_convolve2
        _check(self.ctx.ptr, fn(self.ptr, C.byref(a), C.byref(b), o.grid.ptr, o.kind, o.x))

    # BaseConvolver API (convolution.hh:74-292)
    def convolve_Gradients(self, inl, d1l, inr, d1r, o, invlap=False):
        self._c2(_opnd(inl, L.MF_OPND_GRAD, d1l), _opnd(inr, L.MF_OPND_GRAD, d1r), o, invlap)

    def convolve_Hessians(self, inl, d2l, inm, d2m, *rest, invlap=False):
        if len(rest) == 1:
            self._c2(_opnd(inl, L.MF_OPND_HESS, d2l), _opnd(inm, L.MF_OPND_HESS, d2m), rest[0], invlap)
        else:
            inr, d2r, o = rest
            a, b, c = (_opnd(inl, L.MF_OPND_HESS, d2l), _opnd(inm, L.MF_OPND_HESS, d2m),
                       _opnd(inr, L.MF_OPND_HESS, d2r))
            _check(self.ctx.ptr, lib().mf_conv_convolve3(self.ptr, C.byref(a), C.byref(b), C.byref(c),
                                                         o.grid.ptr, o.kind, o.x))

    def convolve_SumOfHessians(self, inl, d2l, inr, d2r1, d2r2, o, invlap=False):
        self._c2(_opnd(inl, L.MF_OPND_HESS, d2l), _opnd(inr, L.MF_OPND_SUM, tuple(d2r1) + tuple(d2r2)), o, invlap)

    def convolve_DifferenceOfHessians(self, inl, d2l, inr, d2r1, d2r2, o, invlap=False):
        self._c2(_opnd(inl, L.MF_OPND_HESS, d2l), _opnd(inr, L.MF_OPND_DIFF, tuple(d2r1) + tuple(d2r2)), o, invlap)

    def multiply_field(self, inl, inr, o):
        self._c2(_opnd(inl, L.MF_OPND_PLAIN), _opnd(inr, L.MF_OPND_PLAIN), o)

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_conv_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OrszagConvolver(_Convolver):
    KIND = L.MF_CONV_ORSZAG


class NaiveConvolver(_Convolver):
    KIND = L.MF_CONV_NAIVE
