"""CPU oracle for the monofonIC nLPT field pipeline (test infrastructure only).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  It restates, in numpy float64, the reference's own algorithm for the path
white noise -> phi(1) -> Orszag-3/2 convolutions -> phi(2), phi(3), A(3) ->
displacements, velocities, lattice positions and particle IDs.  Every function
cites the reference file:line it follows (paths relative to the monofonIC
source tree).

Parity status: UNPINNED.  The reference ships no golden vectors, known-answer
tests or fixtures for this path, and it cannot be compiled as shipped in this
environment (it needs FFTW3, GSL, HDF5 and a CMake-generated
``cmake_config.hh``).  Third-party arithmetic on the path is FFTW3 (unpinned
version) for the transforms and GSL (unpinned) for the sigma_8 quadrature and
cubic splines; this restatement uses numpy's pocketfft for the transforms
(same sign and Hermitian-input conventions as FFTW's r2c/c2r, see ``c2r``) and
scipy's QUADPACK for the sigma_8 integral.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# ----------------------------------------------------------------------------
# physical constants  (include/physical_constants.hh:24-63)
# ----------------------------------------------------------------------------
_PI = 3.141592653589793115997963468544185161590576171875
MPC_SI = 3.0857e22
C_SI = 2.99792458e8
G_SI = 6.6740800e-11
KB_SI = 1.38064852e-23
HBAR_SI = 1.054571800e-34
SIGMA_SI = (_PI * _PI) * (KB_SI ** 4) / 60.0 / (HBAR_SI ** 3) / (C_SI * C_SI)
RHOCRIT_H2_SI = 3 * 1e10 / (8 * _PI * G_SI) / MPC_SI / MPC_SI

# default parameter set used for unspecified keys
# (src/cosmology_parameters.cc:89-104, selected at include/cosmology_parameters.hh:87)
_DEFAULTS = dict(h=0.67742, Omega_m=0.3099, Omega_b=0.048891054, Omega_DE=0.6901,
                 w_0=-1.0, w_a=0.0, n_s=0.96822, A_s=2.1064e-9, k_p=0.05,
                 YHe=0.245421, N_ur=2.046, m_nu1=0.06, m_nu2=0.0, m_nu3=0.0,
                 Tcmb=2.7255)


def cosmo_parameters(Omega_m, Omega_b, h, sigma_8, n_s, Omega_L=None, Tcmb=None,
                     m_nu1=None, N_ur=None, zero_radiation=False, w_0=None, w_a=None):
    """Derived cosmological parameters, ``ParameterSet = none`` branch.

    Follows include/cosmology_parameters.hh:84-196 (reading with defaults,
    derived radiation densities, flatness closure through Omega_DE).
    """
    d = _DEFAULTS
    p = {}
    p["Tcmb"] = d["Tcmb"] if Tcmb is None else Tcmb
    p["h"] = h
    p["n_s"] = n_s
    p["sigma_8"] = sigma_8
    p["A_s"] = -1.0
    p["k_p"] = d["k_p"]
    p["Omega_b"] = Omega_b
    p["Omega_m"] = Omega_m
    p["m_nu1"] = d["m_nu1"] if m_nu1 is None else m_nu1
    p["m_nu2"] = d["m_nu2"]
    p["m_nu3"] = d["m_nu3"]
    n_nu_massive = int(p["m_nu1"] > 1e-9) + int(p["m_nu2"] > 1e-9) + int(p["m_nu3"] > 1e-9)
    p["N_ur"] = (3.046 - n_nu_massive) if N_ur is None else N_ur
    p["Omega_DE"] = d["Omega_DE"] if Omega_L is None else Omega_L
    p["w_0"] = d["w_0"] if w_0 is None else w_0
    p["w_a"] = d["w_a"] if w_a is None else w_a
    p["H0"] = 100.0 * h
    sum_m_nu = p["m_nu1"] + p["m_nu2"] + p["m_nu3"]
    p["Omega_nu_massive"] = sum_m_nu / (93.14 * h * h)
    p["Omega_gamma"] = (4 * SIGMA_SI / C_SI ** 3 * p["Tcmb"] ** 4.0
                        / RHOCRIT_H2_SI / (h * h))
    p["Omega_nu_massless"] = p["N_ur"] * p["Omega_gamma"] * 7. / 8. * (4. / 11.) ** (4. / 3.)
    p["Omega_r"] = p["Omega_gamma"] + p["Omega_nu_massless"]
    p["Omega_c"] = p["Omega_m"] - p["Omega_b"] - p["Omega_nu_massive"]
    if zero_radiation:
        p["Omega_r"] = 0.0
    p["f_b"] = p["Omega_b"] / p["Omega_m"]
    p["f_c"] = 1.0 - p["f_b"]
    p["Omega_DE"] += 1.0 - p["Omega_m"] - p["Omega_DE"] - p["Omega_r"]
    p["Omega_k"] = 0.0
    return p


# ----------------------------------------------------------------------------
# Eisenstein & Hu (1998) fit  (src/plugins/transfer_eisenstein.cc:58-201)
# ----------------------------------------------------------------------------
class EisensteinHu:
    """E&H 'full' transfer-function fit; restates TFset_parameters/TFfit_onek."""

    def __init__(self, p):
        # set_parameters (transfer_eisenstein.cc:186-194)
        H0, Om, Ob, Tcmb = p["H0"], p["Omega_m"], p["Omega_b"], p["Tcmb"]
        self.m_h0 = H0 * 0.01
        self._set(Om * H0 * H0 * (0.01 * 0.01), Ob / Om, Tcmb)
        self.fb = Ob / Om
        self.fc = (Om - Ob) / Om

    def _set(self, omhh, f_baryon, Tcmb):
        # TFset_parameters (transfer_eisenstein.cc:58-122)
        pw = math.pow
        self.omhh = omhh
        self.obhh = omhh * f_baryon
        if Tcmb <= 0.0:
            Tcmb = 2.728
        th = Tcmb / 2.7
        self.z_equality = 2.50e4 * omhh / th ** 4
        self.k_equality = 0.0746 * omhh / th ** 2
        b1 = 0.313 * pw(omhh, -0.419) * (1 + 0.607 * pw(omhh, 0.674))
        b2 = 0.238 * pw(omhh, 0.223)
        self.z_drag = (1291 * pw(omhh, 0.251) / (1 + 0.659 * pw(omhh, 0.828))
                       * (1 + b1 * pw(self.obhh, b2)))
        self.R_drag = 31.5 * self.obhh / th ** 4 * (1000 / (1 + self.z_drag))
        self.R_equality = 31.5 * self.obhh / th ** 4 * (1000 / self.z_equality)
        self.sound_horizon = (2. / 3. / self.k_equality * math.sqrt(6. / self.R_equality)
                              * math.log((math.sqrt(1 + self.R_drag) + math.sqrt(self.R_drag + self.R_equality))
                                         / (1 + math.sqrt(self.R_equality))))
        self.k_silk = 1.6 * pw(self.obhh, 0.52) * pw(omhh, 0.73) * (1 + pw(10.4 * omhh, -0.95))
        a1 = pw(46.9 * omhh, 0.670) * (1 + pw(32.1 * omhh, -0.532))
        a2 = pw(12.0 * omhh, 0.424) * (1 + pw(45.0 * omhh, -0.582))
        self.alpha_c = pw(a1, -f_baryon) * pw(a2, -f_baryon ** 3)
        bb1 = 0.944 / (1 + pw(458 * omhh, -0.708))
        bb2 = pw(0.395 * omhh, -0.0266)
        self.beta_c = 1.0 / (1 + bb1 * (pw(1 - f_baryon, bb2) - 1))
        y = self.z_equality / (1 + self.z_drag)
        G = y * (-6. * math.sqrt(1 + y) + (2. + 3. * y) * math.log((math.sqrt(1 + y) + 1) / (math.sqrt(1 + y) - 1)))
        self.alpha_b = 2.07 * self.k_equality * self.sound_horizon * pw(1 + self.R_drag, -0.75) * G
        self.beta_node = 8.41 * pw(omhh, 0.435)
        self.beta_b = 0.5 + f_baryon + (3. - 2. * f_baryon) * math.sqrt(pw(17.2 * omhh, 2.0) + 1)

    def onek(self, k):
        """TFfit_onek (transfer_eisenstein.cc:125-178), vectorised; returns (T_b, T_c)."""
        k = np.abs(np.asarray(k, dtype=np.float64))
        zero = k == 0.0
        k = np.where(zero, 1.0, k)
        q = k / 13.41 / self.k_equality
        xx = k * self.sound_horizon
        ln_beta = np.log(2.718282 + 1.8 * self.beta_c * q)
        ln_nobeta = np.log(2.718282 + 1.8 * q)
        C_alpha = 14.2 / self.alpha_c + 386.0 / (1 + 69.9 * q ** 1.08)
        C_noalpha = 14.2 + 386.0 / (1 + 69.9 * q ** 1.08)
        f = 1.0 / (1.0 + (xx / 5.4) ** 4)
        T_c = (f * ln_beta / (ln_beta + C_noalpha * q * q)
               + (1 - f) * ln_beta / (ln_beta + C_alpha * q * q))
        s_tilde = self.sound_horizon * (1. + (self.beta_node / xx) ** 3) ** (-1. / 3.)
        xt = k * s_tilde
        T_b_T0 = ln_nobeta / (ln_nobeta + C_noalpha * q * q)
        T_b = np.sin(xt) / xt * (T_b_T0 / (1. + (xx / 5.2) ** 2)
                                 + self.alpha_b / (1. + (self.beta_b / xx) ** 3)
                                 * np.exp(-(k / self.k_silk) ** 1.4))
        T_b = np.where(zero, 1.0, T_b)
        T_c = np.where(zero, 1.0, T_c)
        return T_b, T_c

    def at_k(self, k):
        """at_k (transfer_eisenstein.cc:196-201): k in h/Mpc."""
        tb, tc = self.onek(np.asarray(k, dtype=np.float64) * self.m_h0)
        return self.fb * tb + self.fc * tc


# ----------------------------------------------------------------------------
# growth factor and normalisation (include/cosmology_calculator.hh:91-463)
# ----------------------------------------------------------------------------
def _H_of_a(p, a):
    # cosmology_calculator.hh:317-325
    HH2 = (p["Omega_r"] / (a * a * a * a) + p["Omega_m"] / (a * a * a) + p["Omega_k"] / (a * a)
           + p["Omega_DE"] * a ** (-3. * (1. + p["w_0"] + p["w_a"])) * math.exp(-3. * (1.0 - a) * p["w_a"]))
    return p["H0"] * math.sqrt(HH2)


_CK = dict(a2=0.20, a3=0.30, a4=0.60, a5=1.0, a6=0.8750,
           b21=0.20, b31=3.0 / 40.0, b32=9.0 / 40.0, b41=0.30, b42=-0.90, b43=1.20,
           b51=-11.0 / 54.0, b52=2.50, b53=-70.0 / 27.0, b54=35.0 / 27.0,
           b61=1631.0 / 55296.0, b62=175.0 / 512.0, b63=575.0 / 13824.0, b64=44275.0 / 110592.0,
           b65=253.0 / 4096.0, c1=37.0 / 378.0, c3=250.0 / 621.0, c4=125.0 / 594.0, c6=512.0 / 1771.0)
_CK["dc1"] = _CK["c1"] - 2825.0 / 27648.0
_CK["dc3"] = _CK["c3"] - 18575.0 / 48384.0
_CK["dc4"] = _CK["c4"] - 13525.0 / 55296.0
_CK["dc5"] = -277.0 / 14336.0
_CK["dc6"] = _CK["c6"] - 0.250


def _growth_table(p):
    """compute_growth (cosmology_calculator.hh:91-151) with the Cash-Karp
    quality-controlled stepper of include/math/ode_integrate.hh:39-111."""
    Om, H0 = p["Omega_m"], p["H0"]

    def rhs(y):
        a, D, Dp = y
        Ha = _H_of_a(p, a)
        return np.array([a * a * Ha, Dp, -a * Ha * Dp + 1.5 * Om * H0 ** 2 * D / a])

    a0 = 1e-10
    y = np.array([a0, a0, 2.0 * a0 * _H_of_a(p, a0) / C_SI ** 2])
    t = 1.0 / (a0 * _H_of_a(p, a0))
    dt = 1e-9
    eps = 1e-10
    c = _CK
    ta, tD, tf = [], [], []
    while y[0] < 2.0:
        yscale = np.abs(y) + dt * np.abs(rhs(y))
        h = dt
        # rk_step_qs advances its trial state ytemp in place and retries a
        # rejected step from the state that trial left behind
        # (include/math/ode_integrate.hh:73-110: ytemp is not reset)
        ytmp = y.copy()
        while True:
            base = ytmp
            k1 = h * rhs(base)
            k2 = h * rhs(base + c["b21"] * k1)
            k3 = h * rhs(base + c["b31"] * k1 + c["b32"] * k2)
            k4 = h * rhs(base + c["b41"] * k1 + c["b42"] * k2 + c["b43"] * k3)
            k5 = h * rhs(base + c["b51"] * k1 + c["b52"] * k2 + c["b53"] * k3 + c["b54"] * k4)
            k6 = h * rhs(base + c["b61"] * k1 + c["b62"] * k2 + c["b63"] * k3 + c["b64"] * k4 + c["b65"] * k5)
            ytmp = base + c["c1"] * k1 + c["c3"] * k3 + c["c4"] * k4 + c["c6"] * k6
            yerr = c["dc1"] * k1 + c["dc3"] * k3 + c["dc4"] * k4 + c["dc5"] * k5 + c["dc6"] * k6
            errmax = float(np.max(np.abs(yerr / yscale))) / eps
            if errmax > 1.0:
                h *= max(0.1, 0.9 * errmax ** -0.25)
                continue
            hnext = h * 0.9 * errmax ** -0.2 if errmax > 1.89e-4 else 5 * h
            t += h
            y = ytmp
            break
        ta.append(y[0]); tD.append(y[1]); tf.append(y[2])
        dt = hnext
    ta = np.array(ta); tD = np.array(tD); tf = np.array(tf)
    tf = tf / (ta * np.array([_H_of_a(p, a) for a in ta]) * tD)
    return ta, tD, tf


class _LogLogSpline:
    """interpolated_function_1d<true,true,false> (include/math/interpolate.hh:29-103):
    natural cubic spline of log(y) against log(x) (GSL cspline)."""

    def __init__(self, x, y):
        from scipy.interpolate import CubicSpline
        self.s = CubicSpline(np.log(x), np.log(y), bc_type="natural")

    def __call__(self, x):
        return float(np.exp(self.s(math.log(x))))


@dataclass
class CosmoScalars:
    """Host scalars that cross the boundary: D+(a_start), vfac, sqrt(pnorm)."""
    Dplus: float
    vfac: float
    pnorm: float
    n_s: float
    params: dict = field(default_factory=dict)


def scalars_from(p, Dplus, vfac, pnorm):
    """CosmoScalars sharing externally computed D+, vfac and pnorm (the
    scalars cross the boundary from one host calculator to both sides)."""
    return CosmoScalars(Dplus=Dplus, vfac=vfac, pnorm=pnorm, n_s=p["n_s"], params=p)


def cosmo_calculator(p, zstart):
    """cosmology::calculator ctor (cosmology_calculator.hh:166-210) plus
    get_growth_factor/get_vfact (:334-363) and compute_pnorm_from_sigma8 (:439-463)."""
    from scipy.integrate import quad
    ta, tD, tf = _growth_table(p)
    D_of_a = _LogLogSpline(ta, tD)
    f_of_a = _LogLogSpline(ta, tf)
    Dnow = D_of_a(1.0)
    astart = 1.0 / (1.0 + zstart)
    Dplus = D_of_a(astart) / Dnow
    vfac = f_of_a(astart) * astart * _H_of_a(p, astart) / p["h"]
    eh = EisensteinHu(p)
    ns = p["n_s"]

    def dsigma8(k):  # dSigma8 (cosmology_calculator.hh:368-380)
        x = k * 8.0
        w = 1.0 - 0.1 * x * x if x < 0.001 else 3.0 * (math.sin(x) - x * math.cos(x)) / (x * x * x)
        tfk = float(eh.at_k(k))
        return k * k * w * w * k ** ns * tfk * tfk

    # GSL QAG-61 to rel 1e-10 over [kmin, kmax] = [1e-4, 1e4]
    # (cosmology_calculator.hh:62-83, 439-452); QUADPACK over log-spaced pieces here
    import warnings
    edges = np.logspace(-4, 4, 161)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        sig = sum(quad(dsigma8, a, b, epsabs=0, epsrel=1e-12, limit=400)[0]
                  for a, b in zip(edges[:-1], edges[1:]))
    sigma8_meas = math.sqrt(4.0 * math.pi * sig)
    pnorm = p["sigma_8"] ** 2 / sigma8_meas ** 2
    return CosmoScalars(Dplus=Dplus, vfac=vfac, pnorm=pnorm, n_s=ns, params=p)


# ----------------------------------------------------------------------------
# white noise: project RNG plugin (Philox4x32-10 + Box-Muller), keyed by cell
# ----------------------------------------------------------------------------
_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(ctr, key):
    """Philox4x32-10 (Salmon et al. 2011), vectorised on uint64 lanes."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint64) & _MASK for c in ctr)
    k0, k1 = np.uint64(key[0]) & _MASK, np.uint64(key[1]) & _MASK
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & _MASK, lo1, (hi0 ^ c3 ^ k1) & _MASK, lo0
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def white_noise(n, seed):
    """Real-space i.i.d. N(0,1) float64 noise on an n^3 grid.

    Cell c = (i*n + j)*n + k takes draw c of a stream in which pair
    p = c // 2 is one Philox4x32-10 block at counter (p_lo, p_hi, 0, 0) and key
    (seed_lo, seed_hi); two 53-bit uniforms u1, u2 in (0,1) go through
    Box-Muller: cell 2p gets r cos(2 pi u2), cell 2p+1 gets r sin(2 pi u2).
    This plays the role of RNG_plugin::Fill_Grid (include/random_plugin.hh:37).
    """
    ncell = n * n * n
    npair = (ncell + 1) // 2
    p = np.arange(npair, dtype=np.uint64)
    x0, x1, x2, x3 = philox4x32((p & _MASK, p >> np.uint64(32), 0 * p, 0 * p),
                                (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF))
    b1 = (x0 | (x1 << np.uint64(32))) >> np.uint64(11)
    b2 = (x2 | (x3 << np.uint64(32))) >> np.uint64(11)
    u1 = (b1.astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u2 = (b2.astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    r = np.sqrt(-2.0 * np.log(u1))
    th = 2.0 * math.pi * u2
    out = np.empty(2 * npair)
    out[0::2] = r * np.cos(th)
    out[1::2] = r * np.sin(th)
    return out[:ncell].reshape(n, n, n)


# ----------------------------------------------------------------------------
# Grid_FFT essentials (include/grid_fft.hh, src/grid_fft.cc)
# ----------------------------------------------------------------------------
_FFT_WORKERS = 1


def set_fft_workers(n: int):
    """Threads for the oracle's transforms (the reference's FFTW threads,
    src/main.cc:156-174); >1 switches to scipy's multithreaded pocketfft."""
    global _FFT_WORKERS
    _FFT_WORKERS = max(1, int(n))


def _rfftn(x):
    if _FFT_WORKERS > 1:
        import scipy.fft as sf
        return sf.rfftn(x, axes=(0, 1, 2), workers=_FFT_WORKERS)
    return np.fft.rfftn(x, axes=(0, 1, 2))


def _irfftn(X, n):
    if _FFT_WORKERS > 1:
        import scipy.fft as sf
        return sf.irfftn(X, s=(n, n, n), axes=(0, 1, 2), workers=_FFT_WORKERS)
    return np.fft.irfftn(X, s=(n, n, n), axes=(0, 1, 2))


def r2c(x):
    """FourierTransformForward + ApplyNorm (grid_fft.cc:199-235): FFTW r2c
    (sign -1) of an n^3 real array, scaled by 1/sqrt(n^3)."""
    n = x.shape[0]
    return _rfftn(x) / math.sqrt(float(n) ** 3)


def c2r(X, n=None):
    """FourierTransformBackward + ApplyNorm (grid_fft.cc:238-270): FFTW c2r
    (sign +1) scaled by 1/sqrt(n^3).  For spectra that are not Hermitian on the
    kz = 0 and kz = n/2 planes the result is that of complex inverse
    transforms along x and y followed by a c2r along z that ignores the
    imaginary parts of the kz = 0 and kz = n/2 terms -- FFTW's convention,
    and numpy's irfftn."""
    if n is None:
        n = X.shape[0]
    return _irfftn(X, n) * (float(n) ** 3 / math.sqrt(float(n) ** 3))


def kvec_1d(n, L):
    """get_k per axis (grid_fft.hh:281-296): (i - n*[i > n/2]) * 2pi/L (Nyquist stays +)."""
    i = np.arange(n, dtype=np.float64)
    return (i - (i > n // 2) * n) * (2.0 * math.pi / L)


def grad_1d(n, L):
    """gradient factor (grid_fft.hh:376-385, operators.hh:49-55): real part of
    i*k per axis, zero at the Nyquist index."""
    g = kvec_1d(n, L)
    g[n // 2] = 0.0
    return g


def kgrids(n, L):
    k1 = kvec_1d(n, L)
    kz = k1[: n // 2 + 1]
    return k1[:, None, None], k1[None, :, None], kz[None, None, :]


def ggrids(n, L):
    g1 = grad_1d(n, L)
    gz = g1[: n // 2 + 1]
    return [g1[:, None, None], g1[None, :, None], gz[None, None, :]]


def hessian(F, L, a, b):
    """kfunc of BaseConvolver::convolve_Hessians (convolution.hh:137-160):
    (i g_a)(i g_b) F = -g_a g_b F."""
    n = F.shape[0]
    g = ggrids(n, L)
    return -(g[a] * g[b]) * F


def sum_hessian(F, L, d1, d2, sign=+1):
    """kfunc of convolve_SumOfHessians / DifferenceOfHessians (convolution.hh:214-274)."""
    n = F.shape[0]
    g = ggrids(n, L)
    return (-(g[d1[0]] * g[d1[1]]) + sign * -(g[d2[0]] * g[d2[1]])) * F


# ----------------------------------------------------------------------------
# Orszag 3/2 convolver (include/convolution.hh:429-669)
# ----------------------------------------------------------------------------
def pad_insert(Fk, N):
    """OrszagConvolver::pad_insert (convolution.hh:570-592)."""
    M = 3 * N // 2
    fp = np.zeros((M, M, M // 2 + 1), dtype=np.complex128)
    rfac = math.pow(1.5, 1.5)
    ip = np.arange(N)
    ip = np.where(ip > N // 2, ip + N // 2, ip)
    fp[np.ix_(ip, ip, np.arange(N // 2 + 1))] = Fk * rfac
    return fp


def unpad(Fp, N):
    """OrszagConvolver::unpad (convolution.hh:618-653): gather, divide by
    sqrt(M^3)/sqrt(N^3), zero every i, j or k == N/2 plane."""
    M = Fp.shape[0]
    rfac = math.sqrt(float(M * M * M)) / math.sqrt(float(N * N * N))
    ip = np.arange(N)
    ip = np.where(ip > N // 2, ip + N // 2, ip)
    out = Fp[np.ix_(ip, ip, np.arange(N // 2 + 1))] / rfac
    out[N // 2, :, :] = 0
    out[:, N // 2, :] = 0
    out[:, :, N // 2] = 0
    return out


def orszag_conv2(A, B):
    """OrszagConvolver::convolve2 (convolution.hh:513-535) on pre-evaluated
    kfunc arrays A, B (N-grid half spectra); returns the unpadded result."""
    N = A.shape[0]
    M = 3 * N // 2
    f1 = c2r(pad_insert(A, N), M)
    f2 = c2r(pad_insert(B, N), M)
    return unpad(r2c(f2 * f1), N)


def orszag_conv3(A, B, C):
    """OrszagConvolver::convolve3 (convolution.hh:543-549): two chained
    convolve2, the intermediate truncated and Nyquist-zeroed."""
    return orszag_conv2(orszag_conv2(A, B), C)


def naive_conv2(A, B):
    """NaiveConvolver::convolve2 (convolution.hh:328-356)."""
    N = A.shape[0]
    return r2c(c2r(B, N) * c2r(A, N))


def naive_conv3(A, B, C):
    """NaiveConvolver::convolve3 (convolution.hh:359-402)."""
    N = A.shape[0]
    return r2c(c2r(B, N) * c2r(A, N) * c2r(C, N))


# output operators (include/operators.hh:25-35), applied per real scalar;
# elementwise on complex arrays they are the same arithmetic
def op_apply(target, value, kind, x=1.0):
    if kind == "assign":
        target[...] = value
    elif kind == "add":
        target += value
    elif kind == "sub":
        target -= value
    elif kind == "axpy":
        target += value * x
    else:
        raise ValueError(kind)


def inverse_laplacian(F, L):
    """apply_InverseLaplacian (grid_fft.hh:440-449): -x/k^2 then zero_DC_mode."""
    n = F.shape[0]
    kx, ky, kz = kgrids(n, L)
    k2 = kx * kx + ky * ky + kz * kz
    with np.errstate(divide="ignore", invalid="ignore"):
        out = -F / k2
    out[0, 0, 0] = 0
    return out


# ----------------------------------------------------------------------------
# IC generator LPT section (src/ic_generator.cc:209-563)
# ----------------------------------------------------------------------------
@dataclass
class LPTFields:
    phi: np.ndarray
    phi2: np.ndarray | None
    phi3: np.ndarray | None
    A3: list | None
    wn: np.ndarray | None = None  # normalised k-space white noise (ic_generator.cc:341-346)


def amplitude(kmod, cs, eh):
    """get_amplitude (cosmology_calculator.hh:405-408)."""
    return np.power(kmod, 0.5 * cs.n_s) * eh.at_k(kmod) * math.sqrt(cs.pnorm)


def lpt_potentials(noise_r, L, order, cs, eh=None, convolver="orszag", fixing=False, inversion=False):
    """ic_generator::run, LPT part (ic_generator.cc:249-563 without fNL/tides).

    Returns the growth-scaled potentials phi*g1, phi2*g2, phi3*g3, A3*g3c in
    k-space (n x n x n/2+1 complex each).
    """
    if eh is None:
        eh = EisensteinHu(cs.params)
    conv2 = orszag_conv2 if convolver == "orszag" else naive_conv2
    conv3 = orszag_conv3 if convolver == "orszag" else naive_conv3
    n = noise_r.shape[0]
    volfac = math.pow(L / n / 2.0 / math.pi, 1.5)
    D = cs.Dplus
    g1 = -D
    g2 = -3.0 / 7.0 * D * D if order > 1 else 0.0
    g3 = 1.0 / 3.0 * D * D * D if order > 2 else 0.0
    g3c = 1.0 / 7.0 * D * D * D if order > 2 else 0.0

    wn = r2c(noise_r)
    # normalise (ic_generator.cc:341-346)
    if fixing:
        a = np.abs(wn)
        wn = np.where(a != 0.0, wn / np.where(a != 0, a, 1.0), wn)
    wn = (-1.0 if inversion else 1.0) * wn / volfac
    # phi(1) (ic_generator.cc:449-457)
    kx, ky, kz = kgrids(n, L)
    kmod = np.sqrt(kx * kx + ky * ky + kz * kz)
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = -(wn * amplitude(kmod, cs, eh)) / (kmod * kmod)
    phi[0, 0, 0] = 0

    H = lambda F, a, b: hessian(F, L, a, b)
    phi2 = phi3 = A3 = None
    if order > 1:
        # ic_generator.cc:471-475
        s = conv2(H(phi, 0, 0), sum_hessian(phi, L, (1, 1), (2, 2)))
        s = s + conv2(H(phi, 1, 1), H(phi, 2, 2))
        s = s - conv2(H(phi, 0, 1), H(phi, 0, 1))
        s = s - conv2(H(phi, 0, 2), H(phi, 0, 2))
        s = s - conv2(H(phi, 1, 2), H(phi, 1, 2))
        phi2 = inverse_laplacian(s, L)
    if order > 2:
        # 3a (ic_generator.cc:511-515)
        t = conv3(H(phi, 0, 0), H(phi, 1, 1), H(phi, 2, 2))
        t = t + conv3(H(phi, 0, 1), H(phi, 0, 2), H(phi, 1, 2)) * 2.0
        t = t - conv3(H(phi, 1, 2), H(phi, 1, 2), H(phi, 0, 0))
        t = t - conv3(H(phi, 0, 2), H(phi, 0, 2), H(phi, 1, 1))
        t = t - conv3(H(phi, 0, 1), H(phi, 0, 1), H(phi, 2, 2))
        # 3b (ic_generator.cc:522-527)
        t = t + conv2(H(phi, 0, 0), sum_hessian(phi2, L, (1, 1), (2, 2))) * (-5.0 / 7.0)
        t = t + conv2(H(phi, 1, 1), sum_hessian(phi2, L, (2, 2), (0, 0))) * (-5.0 / 7.0)
        t = t + conv2(H(phi, 2, 2), sum_hessian(phi2, L, (0, 0), (1, 1))) * (-5.0 / 7.0)
        t = t + conv2(H(phi, 0, 1), H(phi2, 0, 1)) * (+10.0 / 7.0)
        t = t + conv2(H(phi, 0, 2), H(phi2, 0, 2)) * (+10.0 / 7.0)
        t = t + conv2(H(phi, 1, 2), H(phi2, 1, 2)) * (+10.0 / 7.0)
        phi3 = inverse_laplacian(t, L)
        # A(3) (ic_generator.cc:534-545)
        A3 = []
        for d in range(3):
            dp, dpp = (d + 1) % 3, (d + 2) % 3
            a = conv2(H(phi2, d, dp), H(phi, d, dpp))
            a = a - conv2(H(phi2, d, dpp), H(phi, d, dp))
            a = a + conv2(H(phi, dp, dpp), sum_hessian(phi2, L, (dp, dp), (dpp, dpp), sign=-1))
            a = a - conv2(H(phi2, dp, dpp), sum_hessian(phi, L, (dp, dp), (dpp, dpp), sign=-1))
            A3.append(inverse_laplacian(a, L))
    # growth scaling (ic_generator.cc:550-563)
    phi = phi * g1
    if order > 1:
        phi2 = phi2 * g2
    if order > 2:
        phi3 = phi3 * g3
        A3 = [a * g3c for a in A3]
    return LPTFields(phi, phi2, phi3, A3, wn)


# ----------------------------------------------------------------------------
# displacement / velocity assembly and the particle lattice
# (src/ic_generator.cc:794-948, include/particle_generator.hh)
# ----------------------------------------------------------------------------
LATTICE_SHIFTS = {  # particle_generator.hh:47-54
    0: [(0.0, 0.0, 0.0)],
    1: [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5)],
    2: [(0.0, 0.0, 0.0), (0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)],
    3: [(0.0, 0.0, 0.0), (0.0, 0.0, 0.5), (0.0, 0.5, 0.0), (0.0, 0.5, 0.5),
        (0.5, 0.0, 0.0), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0), (0.5, 0.5, 0.5)],
}


def displacement_k(f: LPTFields, L, d, order, unit=1.0, vel=False, vfac=0.0, vcorr=None):
    """k-space combination of ic_generator.cc:829-858 (positions) or
    :884-931 (velocities), times unit/L, DC zeroed, with the fourier_gradient
    operator of operators.hh:38-61 (or a PLT gradient passed as ``vcorr``)."""
    n = f.phi.shape[0]
    g = ggrids(n, L)
    dp, dpp = (d + 1) % 3, (d + 2) % 3
    if not vel:
        tot = f.phi.copy()
        if order > 1:
            tot = tot + f.phi2
        if order > 2:
            tot = tot + f.phi3
        t = (1j * g[d]) * tot
        if order > 2:
            t = t + ((1j * g[dp]) * f.A3[dpp] - (1j * g[dpp]) * f.A3[dp])
    else:
        tot = vfac * f.phi
        if order > 1:
            tot = tot + 2 * vfac * f.phi2
        if order > 2:
            tot = tot + 3 * vfac * f.phi3
        t = (1j * g[d]) * tot
        if order > 2:
            t = t + 3 * vfac * ((1j * g[dp]) * f.A3[dpp] - (1j * g[dpp]) * f.A3[dp])
        if vcorr is not None:
            t = t * vcorr
    t = t * (unit / L)
    t[0, 0, 0] = 0
    return t


def shift_field(fr, s, L):
    """shift_field (grid_fft.hh:832-842): r2c, times exp(i s.k dx), c2r."""
    n = fr.shape[0]
    F = r2c(fr)
    kx, ky, kz = kgrids(n, L)
    dx = L / n
    F = F * np.exp(1j * (s[0] * kx * dx + s[1] * ky * dx + s[2] * kz * dx))
    return c2r(F, n)


SECOND_LATTICE_SHIFT = {  # particle_generator.hh:56-63
    0: (0.5, 0.5, 0.5), 1: (0.5, 0.5, 0.0), 2: (0.5, 0.5, 0.5), 3: (0.25, 0.25, 0.25)}


def _sublattice_fields(field_r, lattice, L, secondary=False):
    """the field read out on each sub-lattice: the secondary lattice's global
    shift first, then the relative shifts (particle_generator.hh:389-401,
    :510-522, :607-618), each a shift_field round trip"""
    shifts = LATTICE_SHIFTS[lattice]
    fr = field_r
    for ish, s in enumerate(shifts):
        if ish == 0 and secondary:
            fr = shift_field(fr, SECOND_LATTICE_SHIFT[lattice], L)
        if ish > 0:
            prev = shifts[ish - 1]
            fr = shift_field(fr, tuple(s[a] - prev[a] for a in range(3)), L)
        yield ish, s, fr


def lattice_positions_component(field_r, d, lattice, unit, L, secondary=False):
    """set_positions, Bravais branch (particle_generator.hh:499-544), one
    component d: returns the overload*n^3 values pos[ip] in particle order
    ishift*n^3 + cell; the secondary lattice adds second_lattice_shift to q
    (particle_generator.hh:531)."""
    n = field_r.shape[0]
    out = []
    idx = np.arange(n, dtype=np.float64)
    for ish, s, fr in _sublattice_fields(field_r, lattice, L, secondary):
        sd = s[d] + (SECOND_LATTICE_SHIFT[lattice][d] if secondary else 0.0)
        q = (idx + sd) / float(n)
        qg = [q[:, None, None], q[None, :, None], q[None, None, :]][d]
        out.append((qg * unit + fr).reshape(-1))
    return np.concatenate(out)


def lattice_velocities_component(field_r, lattice, L, secondary=False):
    """set_velocities, Bravais branch (particle_generator.hh:597-639)."""
    return np.concatenate([fr.reshape(-1) for _, _, fr in _sublattice_fields(field_r, lattice, L, secondary)])


def particle_ids(n, lattice, id_offset=0):
    """lattice_generator ctor, Bravais branch (particle_generator.hh:212-253):
    particle ipcount + iload*n^3 gets id offset*overload*n^3 + overload*cell + iload."""
    overload = 1 << max(0, lattice)
    ncell = n * n * n
    cell = np.arange(ncell, dtype=np.uint64)
    off = np.uint64(id_offset * overload * ncell)
    ids = np.empty(overload * ncell, dtype=np.uint64)
    for il in range(overload):
        ids[il * ncell:(il + 1) * ncell] = off + np.uint64(overload) * cell + np.uint64(il)
    return ids


def particles(f: LPTFields, L, order, vfac, lattice=0, lunit=1.0, vunit=1.0):
    """Positions (AoS [ip][3]), velocities (AoS) and ids for the Lagrangian
    particle output of ic_generator.cc:794-948."""
    n = f.phi.shape[0]
    overload = 1 << max(0, lattice)
    pos = np.empty((overload * n ** 3, 3))
    vel = np.empty((overload * n ** 3, 3))
    for d in range(3):
        fr = c2r(displacement_k(f, L, d, order, unit=lunit), n)
        pos[:, d] = lattice_positions_component(fr, d, lattice, lunit, L)
    for d in range(3):
        fr = c2r(displacement_k(f, L, d, order, unit=vunit, vel=True, vfac=vfac), n)
        vel[:, d] = lattice_velocities_component(fr, lattice, L)
    return pos, vel, particle_ids(n, lattice)


# ----------------------------------------------------------------------------
# two species: dark matter and baryons (ic_generator.cc:153-166, :608-948)
# ----------------------------------------------------------------------------
def bc_amplitudes(kmod, cs, Tdbc, Ttbc, vrel, Dplus_target=1.0):
    """get_amplitude_delta_bc / get_amplitude_theta_bc
    (cosmology_calculator.hh:416-431); Tdbc, Ttbc callables of k or None (0,
    as the Eisenstein-Hu plugin returns)"""
    zero = lambda k: np.zeros_like(k)
    Td = (Tdbc or zero)(kmod)
    Tt = (Ttbc or zero)(kmod)
    sDr = math.sqrt(Dplus_target / cs.Dplus)
    pk = np.power(kmod, 0.5 * cs.n_s)
    dbc = Td + (2 * Tt * (sDr - 1.0) if vrel else 0.0)
    a_d = pk * dbc * (math.sqrt(cs.pnorm) * Dplus_target)
    a_t = pk * (Tt * sDr) * (math.sqrt(cs.pnorm) * Dplus_target) if vrel else np.zeros_like(kmod)
    return a_d, a_t


def two_species_particles(f: LPTFields, L, order, cs, Omega_m, Omega_b, lattice=0, lunit=1.0, vunit=1.0, munit=1.0,
                          Tdbc=None, Ttbc=None, vrel=False, Dplus_target=1.0):
    """DoBaryons with a particle output plugin: per species (dm, baryon) the
    positions, velocities, ids and masses.  Baryons sit on the secondary
    lattice and take IDoffset 1 (ic_generator.cc:626-637); the masses are
    pmeanmass (1 + C_s delta_bc) Omega_s munit (:641-673, set_masses
    particle_generator.hh:369-422); with DoBaryonVrel the velocities carry
    -vfac C_s amp_tbc wn grad / k^2 (:907-910)."""
    n = f.phi.shape[0]
    overload = 1 << max(0, lattice)
    kx, ky, kz = kgrids(n, L)
    kmod = np.sqrt(kx * kx + ky * ky + kz * kz)
    a_d, a_t = bc_amplitudes(kmod, cs, Tdbc, Ttbc, vrel, Dplus_target)
    rho_k = f.wn * a_d
    rho_k[0, 0, 0] = 0
    delta = c2r(rho_k, n)
    fb = Omega_b / Omega_m
    g = ggrids(n, L)
    out = {}
    for sp, name in enumerate(("dm", "baryon")):
        C = (1.0 - fb) if name == "baryon" else -fb
        Om_s = Omega_b if name == "baryon" else Omega_m - Omega_b
        sec = name == "baryon"
        pos = np.empty((overload * n ** 3, 3))
        vel = np.empty((overload * n ** 3, 3))
        for d in range(3):
            fr = c2r(displacement_k(f, L, d, order, unit=lunit), n)
            pos[:, d] = lattice_positions_component(fr, d, lattice, lunit, L, secondary=sec)
        for d in range(3):
            t = displacement_k(f, L, d, order, unit=vunit, vel=True, vfac=cs.vfac)
            if vrel:
                with np.errstate(divide="ignore", invalid="ignore"):
                    bc = -cs.vfac * C * a_t * f.wn * (1j * g[d]) / (kmod * kmod)
                bc[0, 0, 0] = 0
                t = t + bc * (vunit / L)
            vel[:, d] = lattice_velocities_component(c2r(t, n), lattice, L, secondary=sec)
        rho = (1.0 + C * delta) * Om_s * munit
        pmean = 1.0 / (n ** 3 * overload)
        mass = np.concatenate([pmean * fr.reshape(-1) for _, _, fr in _sublattice_fields(rho, lattice, L, sec)])
        out[name] = (pos, vel, particle_ids(n, lattice, id_offset=sp), mass)
    return out


def _full_kgrids(n, L):
    """get_k over a complex n^3 grid (grid_fft.hh:282-296): index > n/2 negative"""
    idx = np.arange(n)
    k = (idx - (idx > n // 2) * n) * (2.0 * math.pi / L)
    return np.meshgrid(k, k, k, indexing="ij")


def eulerian_fields(f: LPTFields, L, order, cs, C, Tdbc=None, vunit=1.0, Dplus_target=1.0):
    """the semiclassical (PPT) Eulerian branch of a species
    (ic_generator.cc:679-791): returns the density contrast |psi|^2 - 1 and
    the three velocity components"""
    n = f.phi.shape[0]
    kx, ky, kz = kgrids(n, L)
    kmod = np.sqrt(kx * kx + ky * ky + kz * kz)
    a_d, _ = bc_amplitudes(kmod, cs, Tdbc, None, False, Dplus_target)
    rk = f.wn * a_d
    rk[0, 0, 0] = 0
    prho = np.sqrt(1.0 + C * c2r(rk, n))
    phi = c2r(f.phi, n)
    d = np.abs(np.diff(phi, axis=0))  # base i in 0..n-2 (ic_generator.cc:704)
    dy = np.abs(np.roll(phi, -1, axis=1) - phi)[:-1]
    dz = np.abs(np.roll(phi, -1, axis=2) - phi)[:-1]
    maxd = max(d.max(), dy.max(), dz.max())
    D = cs.Dplus
    hbar = maxd / math.pi / D * 1.01
    phi2 = c2r(f.phi2, n) if order > 1 else None
    arg = (phi + phi2) if order > 1 else phi
    psi = prho * np.exp(1j * (1.0 / hbar) * arg / D)
    K = _full_kgrids(n, L)
    k2 = K[0] ** 2 + K[1] ** 2 + K[2] ** 2
    psi = np.fft.ifftn(np.fft.fftn(psi, norm="ortho") * np.exp(-0.5j * hbar * k2 * D), norm="ortho")
    if order > 1:
        psi = psi * np.exp(1j * (1.0 / hbar) * phi2 / D)
    rho = (psi.real ** 2 + psi.imag ** 2) - 1.0
    vu = D * cs.vfac / L * vunit
    psik = np.fft.fftn(psi, norm="ortho")
    vel = []
    for dd in range(3):
        g = np.fft.ifftn(psik * (1j * K[dd]), norm="ortho")
        vel.append(vu * np.real((np.conj(psi) * g - psi * np.conj(g)) / (2j / hbar)) / (1.0 + rho))
    return rho, vel


# ----------------------------------------------------------------------------
# power spectrum (src/grid_fft.cc:1133-1210)
# ----------------------------------------------------------------------------
def power_spectrum(F, L):
    """Compute_PowerSpectrum of a k-space field; returns (k, P, eP, count)."""
    n = F.shape[0]
    kfac = 2.0 * math.pi / L
    kmax = kfac * (n // 2)
    kmin = kfac
    nbins = int(kmax / kmin)
    kx, ky, kz = kgrids(n, L)
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    k = np.broadcast_to(k, F.shape)
    v = F.real ** 2 + F.imag ** 2
    w = np.ones(F.shape)
    w[:, :, 1:] = 2.0
    sel = (k >= kmin) & (k < kmax)
    idx = (k[sel] / kmin).astype(np.int64)
    bk = np.bincount(idx, weights=(w * k)[sel], minlength=nbins)[:nbins]
    bP = np.bincount(idx, weights=(w * v)[sel], minlength=nbins)[:nbins]
    beP = np.bincount(idx, weights=(w * v * v)[sel], minlength=nbins)[:nbins]
    bc = np.bincount(idx, weights=w[sel], minlength=nbins)[:nbins]
    volfac = L ** 3 / (2.0 * math.pi) ** 3
    fftfac = 1.0 / float(n) ** 3
    with np.errstate(divide="ignore", invalid="ignore"):
        bk = np.where(bc > 0, bk / bc, 0)
        bP = np.where(bc > 0, bP / bc * volfac * fftfac, 0)
        beP = np.where(bc > 0, np.sqrt(beP / bc - bP * bP) / np.sqrt(bc) * volfac * fftfac, 0)
    return bk, bP, beP, bc.astype(np.int64)


# ----------------------------------------------------------------------------
# PLT corrections (include/particle_plt.hh:50-587)
# ----------------------------------------------------------------------------
def _plt_lattice(lattice):
    """Bravais / reciprocal / inverse-reciprocal matrices, FBZ normals and
    charge factor (particle_plt.hh:76-164); RSC falls back to SC (:166-172)."""
    pi, twopi, fourpi = math.pi, 2 * math.pi, 4 * math.pi
    if lattice == 1:
        B = np.array([[1, 0, 0.5], [0, 1, 0.5], [0, 0, 0.5]])
        R = np.array([[twopi, 0, 0], [0, twopi, 0], [-twopi, -twopi, fourpi]])
        IR = np.array([[2, 0, 0], [0, 2, 0], [1, 1, 1]])
        nrm = [(0, pi, pi), (0, -pi, pi), (0, pi, -pi), (0, -pi, -pi), (pi, 0, pi), (-pi, 0, pi),
               (pi, 0, -pi), (-pi, 0, -pi), (pi, pi, 0), (-pi, pi, 0), (pi, -pi, 0), (-pi, -pi, 0)]
        cf = 2
    elif lattice == 2:
        B = np.array([[0, 0.5, 0], [0.5, 0, 1], [0.5, 0.5, 0]])
        R = np.array([[-fourpi, fourpi, twopi], [0, 0, twopi], [fourpi, 0, -twopi]])
        IR = np.array([[0, 1, 1], [1, 0, 1], [0, 2, 0]])
        nrm = [(twopi, 0, 0), (-twopi, 0, 0), (0, twopi, 0), (0, -twopi, 0), (0, 0, twopi), (0, 0, -twopi),
               (pi, pi, pi), (pi, pi, -pi), (pi, -pi, pi), (pi, -pi, -pi), (-pi, pi, pi), (-pi, pi, -pi),
               (-pi, -pi, pi), (-pi, -pi, -pi)]
        cf = 4
    else:
        B = np.eye(3)
        R = np.eye(3) * twopi
        IR = np.eye(3, dtype=int) * 2
        nrm = [(pi, 0, 0), (-pi, 0, 0), (0, pi, 0), (0, -pi, 0), (0, 0, pi), (0, 0, -pi)]
        cf = 1
    return B.astype(float), R.astype(float), IR.astype(int), np.array(nrm, dtype=float), cf


def plt_tables(lattice, ng):
    """lattice_gradient::init_D (particle_plt.hh:68-515), vectorised; returns
    the real tables (D_r, D_theta, D_phi, D_vfac) on the (ng, ng, ng/2+1)
    k-space mesh.  Map insertions follow the sequential loop order (first
    insertion of a key wins)."""
    B, R, IR, normals, cf = _plt_lattice(lattice)
    nl = ng
    dx = 1.0 / nl
    eta = 4.0
    alpha = 1.0 / math.sqrt(2) / eta
    a2, a3 = alpha * alpha, alpha ** 3
    charge = 1.0 / nl ** 3 / cf
    fft_norm = 1.0 / nl ** 3.0
    idx = np.arange(nl)
    X = np.stack(np.meshgrid(idx, idx, idx, indexing="ij"), -1).reshape(-1, 3) * dx
    ar = np.fmod(2.0 + X @ B.T, 1.0)
    M = np.zeros((ar.shape[0], 3, 3))
    rng = range(-3, 4)
    for ix in rng:
        for iy in rng:
            for iz in rng:
                d = ar - B @ np.array([ix, iy, iz], dtype=float)
                r = np.sqrt(np.sum(d * d, axis=1))
                ok = r >= 1e-14
                rs = np.where(ok, r, 1.0)
                r2, r3, r5 = rs * rs, rs ** 3, rs ** 5
                K1 = -a3 / math.pi ** 1.5 * np.exp(-a2 * r2) / r2
                from scipy.special import erfc
                K2 = (erfc(alpha * rs) + 2.0 * alpha / math.sqrt(math.pi) * np.exp(-a2 * r2) * rs) / (4 * math.pi)
                dd = d[:, :, None] * d[:, None, :]
                add = dd * K1[:, None, None] + (np.eye(3)[None] / r3[:, None, None] - 3.0 * dd / r5[:, None, None]) * K2[:, None, None]
                M += np.where(ok[:, None, None], add, 0.0)
    for ix in rng:
        for iy in rng:
            for iz in rng:
                if abs(ix) + abs(iy) + abs(iz) == 0:
                    continue
                ak = R @ (np.array([ix, iy, iz], dtype=float) / nl)
                km2 = ak @ ak
                term = np.exp(-km2 / (4 * a2)) * np.cos(ar @ ak) / km2 * fft_norm
                M += np.outer(ak, ak)[None] * term[:, None, None]
    D6 = [M[:, a, b].reshape(nl, nl, nl) * charge for a, b in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))]
    for a, v in enumerate((1.0 / 3, 0.0, 0.0, 1.0 / 3, 0.0, 1.0 / 3)):
        D6[a][0, 0, 0] = v
    Dk = [np.fft.rfftn(f).real for f in D6]  # unitary r2c times nl^1.5 = plain DFT
    nk = nl // 2 + 1
    kc = (np.arange(nl) - (np.arange(nl) > nl // 2) * nl) * 2 * math.pi
    KX, KY, KZ = np.meshgrid(kc, kc, kc[:nk], indexing="ij")
    kv = np.stack([KX, KY, KZ], -1).reshape(-1, 3)
    Dm = np.empty((kv.shape[0], 3, 3))
    for (a, b), f in zip(((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)), Dk):
        Dm[:, a, b] = Dm[:, b, a] = f.reshape(-1)
    ev, V = np.linalg.eigh(Dm)  # ascending
    e3 = V[:, :, 2] / (2 * math.pi * ng)
    T = np.stack([Dk[0].reshape(-1), Dk[1].reshape(-1), Dk[2].reshape(-1), Dk[3].reshape(-1),
                  Dk[4].reshape(-1), Dk[5].reshape(-1)], 1)
    a_vec = (kv / (2 * math.pi * ng)) @ R.T
    shifts = [(l1, l2, l3, s) for l1 in (-1, 0, 1) for l2 in (-1, 0, 1) for l3 in (-1, 0, 1) for s in (-1.0, 1.0)]
    keys_all, q_all, valid_all = [], [], []
    for (l1, l2, l3, sg) in shifts:
        vk = sg * a_vec + R @ np.array([l1, l2, l3], dtype=float)
        ok = np.all(vk @ normals.T <= 1.0001 * np.sum(normals * normals, axis=1)[None], axis=1)
        key = np.round(vk * ng / (2 * math.pi)).astype(np.int64)
        keys_all.append(key)
        valid_all.append(ok)
    keys_all = np.stack(keys_all, 1)  # (nq, nshift, 3)
    valid_all = np.stack(valid_all, 1)
    anyv = valid_all.any(axis=1)
    T[anyv] = np.stack([ev[anyv, 2], ev[anyv, 1], ev[anyv, 0], e3[anyv, 0], e3[anyv, 1], e3[anyv, 2]], 1)
    off, K = 8 * ng, 16 * ng
    enc = lambda k: ((k[..., 0] + off) * K + (k[..., 1] + off)) * K + (k[..., 2] + off)
    flat_keys = enc(keys_all).reshape(-1)
    flat_q = np.repeat(np.arange(kv.shape[0]), len(shifts))
    sel = valid_all.reshape(-1)
    fk, fq = flat_keys[sel], flat_q[sel]
    ukeys, first = np.unique(fk, return_index=True)
    uq = fq[first]

    def lookup(k):
        e = enc(k)
        pos = np.clip(np.searchsorted(ukeys, e), 0, len(ukeys) - 1)
        found = ukeys[pos] == e
        return np.where(found, uq[pos], -1)

    ii = np.arange(nl) - (np.arange(nl) > nl // 2) * nl
    kk = np.arange(nk) - (np.arange(nk) > nl // 2) * nl
    I, J, Kq = np.meshgrid(ii, ii, kk, indexing="ij")
    sgn = np.stack([I, J, Kq], -1).reshape(-1, 3)
    ui, uj, uk = np.meshgrid(np.arange(nl), np.arange(nl), np.arange(nk), indexing="ij")
    uidx = np.stack([ui, uj, uk], -1).reshape(-1, 3)
    isin = np.all((uidx @ IR.T) % 2 == 0, axis=1)
    kvv = sgn.astype(float)

    def align(v):
        return v * np.where(np.sum(v * kvv, axis=1) < 0, -1.0, 1.0)[:, None]

    l = np.zeros((kv.shape[0], 3))
    v = np.zeros((kv.shape[0], 3))
    cnt = np.zeros(kv.shape[0])
    for o in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
        q = lookup(sgn + np.array(o))
        f = (q >= 0) & ~isin
        qq = np.where(q >= 0, q, 0)
        l += np.where(f[:, None], T[qq][:, 0:3], 0.0)
        v += np.where(f[:, None], align(T[qq][:, 3:6]), 0.0)
        cnt += f
    with np.errstate(invalid="ignore", divide="ignore"):
        l = np.where(~isin[:, None], l / cnt[:, None], l)
        v = np.where(~isin[:, None], v / cnt[:, None], v)
    q = lookup(sgn)
    f = isin & (q >= 0)
    qq = np.where(q >= 0, q, 0)
    l = np.where(f[:, None], T[qq][:, 0:3], np.where(isin[:, None], 0.0, l))
    v = np.where(f[:, None], align(T[qq][:, 3:6]), np.where(isin[:, None], 0.0, v))
    mu1 = l[:, 0]
    with np.errstate(invalid="ignore", divide="ignore"):
        e1 = v / np.linalg.norm(v, axis=1)[:, None]
    kr = np.linalg.norm(kv, axis=1)
    kphi = np.where(kr > 0, np.arctan2(kv[:, 1], kv[:, 0]), 0.0)
    kth = np.where(kr > 0, np.arccos(np.where(kr > 0, kv[:, 2] / np.where(kr > 0, kr, 1), 1.0)), 0.0)
    st, ct, sp, cp = np.sin(kth), np.cos(kth), np.sin(kphi), np.cos(kphi)
    e_r = np.stack([st * cp, st * sp, ct], 1)
    e_t = np.stack([ct * cp, ct * sp, -st], 1)
    e_p = np.stack([-sp, cp, 0 * sp], 1)
    ren = np.sum(e1 * e_r, 1)
    ren = np.where(ren < 0.01, 1.0, ren)
    Dr = np.ones(kv.shape[0])
    Dth = np.sum(e1 * e_t, 1) / ren
    Dph = np.sum(e1 * e_p, 1) / ren
    with np.errstate(invalid="ignore", divide="ignore"):
        Dvf = 1.0 / (0.25 * (np.sqrt(1.0 + 24 * mu1) - 1.0))
    Dvf[0], Dr[0], Dth[0], Dph[0] = 1.0, 1.0, 0.0, 0.0
    shp = (nl, nl, nk)
    return Dr.reshape(shp), Dth.reshape(shp), Dph.reshape(shp), Dvf.reshape(shp)


def _cic_kspace(tab, x, y, z):
    """get_cic_kspace (grid_fft.hh:347-373) of a real table, vectorised."""
    ng = tab.shape[0]
    nk = tab.shape[2]
    ix, iy, iz = np.floor(x).astype(int), np.floor(y).astype(int), np.floor(z).astype(int)
    dx, dy, dz = x - ix, y - iy, z - iz
    tx, ty, tz = 1 - dx, 1 - dy, 1 - dz
    ix1, iy1, iz1 = (ix + 1) % ng, (iy + 1) % ng, np.minimum(iz + 1, nk - 1)
    return (tab[ix, iy, iz] * tx * ty * tz + tab[ix, iy, iz1] * tx * ty * dz + tab[ix, iy1, iz] * tx * dy * tz
            + tab[ix, iy1, iz1] * tx * dy * dz + tab[ix1, iy, iz] * dx * ty * tz + tab[ix1, iy, iz1] * dx * ty * dz
            + tab[ix1, iy1, iz] * dx * dy * tz + tab[ix1, iy1, iz1] * dx * dy * dz)


def plt_gradient(tables, n, L):
    """lattice_gradient::gradient / vfac_corr (particle_plt.hh:551-585) on
    the n-grid half spectrum: returns ([g_x, g_y, g_z], vfac_corr) with the
    gradient i*g_d."""
    Dr_t, Dth_t, Dph_t, Dvf_t = tables
    ng = Dr_t.shape[0]
    mr = ng / n
    i = np.arange(n) * mr
    kz_ = np.arange(n // 2 + 1) * mr
    X, Y, Z = np.meshgrid(i, i, kz_, indexing="ij")
    kcomp = lambda a: (a - (a > ng // 2) * ng) * 2 * math.pi
    kx, ky, kz = kcomp(X), kcomp(Y), kcomp(Z)
    kr = np.sqrt(kx * kx + ky * ky + kz * kz)
    kmod = kr / mr / L
    D_r, D_t, D_p = _cic_kspace(Dr_t, X, Y, Z), _cic_kspace(Dth_t, X, Y, Z), _cic_kspace(Dph_t, X, Y, Z)
    kphi = np.where(kr > 0, np.arctan2(ky, kx), 0.0)
    kth = np.where(kr > 0, np.arccos(np.where(kr > 0, kz / np.where(kr > 0, kr, 1), 1.0)), 0.0)
    st, ct, sp, cp = np.sin(kth), np.cos(kth), np.sin(kphi), np.cos(kphi)
    g = [kmod * (D_r * st * cp + D_t * ct * cp - D_p * sp),
         kmod * (D_r * st * sp + D_t * ct * sp + D_p * cp),
         kmod * (D_r * ct - D_t * st)]
    return g, _cic_kspace(Dvf_t, X, Y, Z)


def displacement_k_plt(f: LPTFields, L, d, order, tables, unit=1.0, vel=False, vfac=0.0):
    """ic_generator.cc:829-931 with the PLT lattice_gradient in place of
    op::fourier_gradient (ENABLE_PLT, ic_generator.cc:366-370)."""
    n = f.phi.shape[0]
    g, vc = plt_gradient(tables, n, L)
    dp, dpp = (d + 1) % 3, (d + 2) % 3
    w = [1.0, 1.0, 1.0] if not vel else [vfac, 2 * vfac, 3 * vfac]
    tot = w[0] * f.phi
    if order > 1:
        tot = tot + w[1] * f.phi2
    if order > 2:
        tot = tot + w[2] * f.phi3
    t = (1j * g[d]) * tot
    if order > 2:
        a = (1j * g[dp]) * f.A3[dpp] - (1j * g[dpp]) * f.A3[dp]
        t = t + (3 * vfac if vel else 1.0) * a
    if vel:
        t = t * vc
    t = t * (unit / L)
    t[0, 0, 0] = 0
    return t
