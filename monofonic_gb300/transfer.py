"""Host transfer-function plugins that feed the pipeline's T(k) table.

The pipeline takes T(k) either from its device Eisenstein & Hu fit or from a
host table with one value per integer k^2 = 0 .. 3(N/2)^2 at
k = sqrt(k^2) 2pi/L (``mf_ic_params.tk_table``; for two species also the
baryon-CDM tables ``tk_dbc_table`` / ``tk_tbc_table``).  This module is the
reference's ``CAMB_file`` transfer plugin (src/plugins/transfer_CAMB_file.cc)
restated for that table interface:

- the file: whitespace-separated rows of at least 13 numbers, lines holding a
  ``#`` skipped (transfer_CAMB_file.cc:37-84); column 0 is k [h/Mpc], 1 the
  CDM, 2 the baryon, 5 the massive-neutrino and 6 the total-matter density
  transfer functions, 10 and 11 the CDM and baryon velocity transfer
  functions; the neutrino and matter velocity entries repeat the total-matter
  density column, as the reference stores them (:88-97);
- interpolation: natural cubic splines of log T against log k
  (``interpolated_function_1d<true, true, false>``, include/math/interpolate.hh,
  GSL ``gsl_interp_cspline``), restated here from the published natural-spline
  equations;
- ``compute(k, type)``: k clamped below at the second tabulated k (:152-153);
  above the last tabulated k the spline is undefined and an error is raised;
- sigma_8 normalisation: ``pnorm = (sigma_8 / sigma_8,measured)^2`` with
  sigma_8,measured^2 = 4 pi int_{kmin}^{kmax} k^2 W^2(8k) k^{n_s} T^2 dk over
  [k_1, k_{n-2}] (cosmology_calculator.hh:368-380, 439-463), so a pipeline run
  with the table is normalised as the reference normalises it.
"""
from __future__ import annotations

import math

import numpy as np

from . import ic

# tf_type of include/transfer_function_plugin.hh
TF_TYPES = ("delta_matter", "delta_cdm", "delta_baryon", "theta_matter", "theta_cdm", "theta_baryon", "delta_bc",
            "theta_bc", "delta_matter0", "delta_cdm0", "delta_baryon0", "theta_matter0", "theta_cdm0",
            "theta_baryon0")


class NaturalCubicSpline:
    """y(x) through the points (x_i, y_i) with zero second derivative at both
    ends; the second-derivative system is tridiagonal and solved directly."""

    def __init__(self, x, y):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        n = x.size
        if n < 3 or y.size != n:
            raise ValueError("a spline needs at least three points and as many y as x")
        h = np.diff(x)
        if not np.all(h > 0):
            raise ValueError("spline abscissae must increase strictly")
        slope = np.diff(y) / h
        # c_i = y''(x_i)/2, c_0 = c_{n-1} = 0; rows i = 1 .. n-2:
        # h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1} = 3 (slope_i - slope_{i-1})
        c = np.zeros(n)
        m = n - 2
        diag = 2.0 * (h[:-1] + h[1:])
        rhs = 3.0 * (slope[1:] - slope[:-1])
        sub = h[1:-1].copy()  # coupling of rows i and i+1
        dd, rr = diag.copy(), rhs.copy()
        for i in range(1, m):  # forward elimination
            w = sub[i - 1] / dd[i - 1]
            dd[i] -= w * sub[i - 1]
            rr[i] -= w * rr[i - 1]
        sol = np.empty(m)
        sol[m - 1] = rr[m - 1] / dd[m - 1]
        for i in range(m - 2, -1, -1):
            sol[i] = (rr[i] - sub[i] * sol[i + 1]) / dd[i]
        c[1:-1] = sol
        self.x, self.y, self.c = x, y, c
        self.b = slope - h * (c[1:] + 2.0 * c[:-1]) / 3.0
        self.d = (c[1:] - c[:-1]) / (3.0 * h)

    def __call__(self, xq):
        xq = np.asarray(xq, dtype=np.float64)
        if np.any(xq < self.x[0]) or np.any(xq > self.x[-1]):
            raise ValueError("spline evaluated outside its tabulated range")
        i = np.clip(np.searchsorted(self.x, xq, side="right") - 1, 0, self.x.size - 2)
        dx = xq - self.x[i]
        return self.y[i] + dx * (self.b[i] + dx * (self.c[i] + dx * self.d[i]))


class CAMBTransfer:
    """transfer_CAMB_file_plugin: tabulated CAMB transfer functions."""

    NCOL = 13

    def __init__(self, filename: str):
        rows = []
        with open(filename) as f:
            for lineno, line in enumerate(f, 1):
                if "#" in line:
                    continue
                parts = line.split()
                if not parts:
                    continue
                try:
                    vals = [float(v) for v in parts[: self.NCOL]]
                except ValueError as e:
                    raise ValueError(f"{filename}:{lineno}: not a transfer-function row") from e
                if len(vals) < self.NCOL:
                    raise ValueError(f"{filename}:{lineno}: {len(vals)} columns, {self.NCOL} expected")
                rows.append(vals)
        if len(rows) < 6:
            raise ValueError(f"{filename}: too few transfer-function rows ({len(rows)})")
        t = np.array(rows)
        self.k = t[:, 0]
        cols = {"dc": t[:, 1], "db": t[:, 2], "dn": t[:, 5], "dm": t[:, 6], "tc": t[:, 10], "tb": t[:, 11]}
        cols["tn"] = cols["dm"]
        cols["tm"] = cols["dm"]
        lk = np.log(self.k)
        with np.errstate(invalid="ignore", divide="ignore"):
            self._spl = {name: NaturalCubicSpline(lk, np.log(v)) for name, v in cols.items()}
        self.kmin = float(self.k[1])
        self.kmax = float(self.k[-2])

    def _eval(self, name, k):
        return np.exp(self._spl[name](np.log(k)))

    def compute(self, k, tf_type: str = "delta_matter"):
        """TransferFunction_plugin::compute(k, type) (transfer_CAMB_file.cc:150-189)"""
        if tf_type not in TF_TYPES:
            raise ValueError(f"invalid transfer function type {tf_type!r}")
        k = np.maximum(np.asarray(k, dtype=np.float64), self.kmin)
        base = tf_type[:-1] if tf_type.endswith("0") else tf_type
        if base == "delta_bc":
            return self._eval("db", k) - self._eval("dc", k)
        if base == "theta_bc":
            return self._eval("tb", k) - self._eval("tc", k)
        name = {"delta_matter": "dm", "delta_cdm": "dc", "delta_baryon": "db", "theta_matter": "tm",
                "theta_cdm": "tc", "theta_baryon": "tb"}[base]
        return self._eval(name, k)

    def table(self, ngrid: int, boxlen: float, tf_type: str = "delta_matter") -> np.ndarray:
        """the pipeline's table: T at k = sqrt(k^2) 2pi/L, k^2 = 0 .. 3(N/2)^2"""
        nk2 = 3 * (ngrid // 2) ** 2 + 1
        k = np.sqrt(np.arange(nk2, dtype=np.float64)) * (2.0 * math.pi / boxlen)
        return np.ascontiguousarray(self.compute(k, tf_type), dtype=np.float64)

    def sigma8(self, n_s: float) -> float:
        """sigma_8 of the unnormalised spectrum k^{n_s} T^2 (compute_sigma8,
        cosmology_calculator.hh:439-453)"""
        from scipy.integrate import quad

        def dsigma8(k):
            x = 8.0 * k
            w = 1.0 - 0.1 * x * x if x < 0.001 else 3.0 * (math.sin(x) - x * math.cos(x)) / (x * x * x)
            t = float(self.compute(k))
            return k * k * w * w * k ** n_s * t * t

        # integrate between the table's nodes, where the spline is smooth
        nodes = self.k[(self.k >= self.kmin) & (self.k <= self.kmax)]
        edges = np.unique(np.concatenate(([self.kmin], nodes, [self.kmax])))
        total = sum(quad(dsigma8, a, b, epsabs=0.0, epsrel=1e-10, limit=200)[0] for a, b in zip(edges[:-1], edges[1:]))
        return math.sqrt(4.0 * math.pi * total)

    def scalars(self, cosmo: "ic.Cosmology", zstart: float):
        """the cosmology scalars with the power spectrum normalised to sigma_8
        through this table (compute_pnorm_from_sigma8, :459-463)"""
        sc = ic.cosmology_scalars(cosmo, zstart)
        sc.sigma8_measured = self.sigma8(cosmo.n_s)
        sc.pnorm = cosmo.sigma_8 ** 2 / sc.sigma8_measured ** 2
        return sc
