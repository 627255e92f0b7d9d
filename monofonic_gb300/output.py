"""Output plugins (include/output_plugin.hh) over libmfgpu's C ABI
(include/monofonic_gb300_output.h): the GRAFIC-2 / RAMSES field writer of
src/plugins/output_grafic2.cc with the plugin's method names."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import Context, Grid_FFT, lib, _check

SPECIES = {"dm": L.MF_SPECIES_DM, "baryon": L.MF_SPECIES_BARYON, "neutrino": L.MF_SPECIES_NEUTRINO}
COMPONENTS = {"density": L.MF_FC_DENSITY, "vx": L.MF_FC_VX, "vy": L.MF_FC_VY, "vz": L.MF_FC_VZ,
              "dx": L.MF_FC_DX, "dy": L.MF_FC_DY, "dz": L.MF_FC_DZ, "mass": L.MF_FC_MASS}
OUTPUT_TYPES = {L.MF_OUTTYPE_PARTICLES: "particles", L.MF_OUTTYPE_FIELD_LAGRANGIAN: "field_lagrangian",
                L.MF_OUTTYPE_FIELD_EULERIAN: "field_eulerian"}


class Grafic2Output:
    """grafic2_output_plugin (output_grafic2.cc:36-136): the constructor makes
    the directory and writes ramses.nml; write_grid_data writes one component
    file from a device field."""

    def __init__(self, ctx: Context, dirname: str, ngrid: int, boxlen: float, zstart: float, H0: float,
                 Omega_m: float, Omega_DE: float, Omega_b: float, baryons: bool = False,
                 ramses_nml: bool = True, use_spt: bool = False, chunk_planes: int = 0):
        self.ctx = ctx
        self._dir = dirname.encode()
        p = L.mf_grafic2_params()
        p.dirname = self._dir
        p.ngrid, p.boxlen, p.zstart, p.H0 = int(ngrid), float(boxlen), float(zstart), float(H0)
        p.Omega_m, p.Omega_DE, p.Omega_b = float(Omega_m), float(Omega_DE), float(Omega_b)
        p.baryons, p.ramses_nml, p.use_spt = int(baryons), int(ramses_nml), int(use_spt)
        p.chunk_planes = int(chunk_planes)
        self.params = p
        h = C.c_void_p()
        _check(ctx.ptr, lib().mf_grafic2_create(ctx.ptr, C.byref(p), C.byref(h)))
        self.ptr = h

    def _info(self, species="dm"):
        wa, r64, i64 = C.c_int(), C.c_int(), C.c_int()
        lu, vu, mu = C.c_double(), C.c_double(), C.c_double()
        _check(self.ctx.ptr, lib().mf_grafic2_info(self.ptr, SPECIES[species], C.byref(wa), C.byref(r64), C.byref(i64),
                                                   C.byref(lu), C.byref(vu), C.byref(mu)))
        return wa.value, bool(r64.value), bool(i64.value), lu.value, vu.value, mu.value

    def write_species_as(self, species: str) -> str:
        return OUTPUT_TYPES[self._info(species)[0]]

    def has_64bit_reals(self) -> bool:
        return self._info()[1]

    def has_64bit_ids(self) -> bool:
        return self._info()[2]

    def position_unit(self) -> float:
        return self._info()[3]

    def velocity_unit(self) -> float:
        return self._info()[4]

    def mass_unit(self) -> float:
        return self._info()[5]

    def write_grid_data(self, g: Grid_FFT, species: str, component: str):
        """write_grid_data(g, s, c) of a real-space Grid_FFT"""
        _check(self.ctx.ptr, lib().mf_grafic2_write_grid(self.ptr, g.ptr, SPECIES[species], COMPONENTS[component]))

    def write_field(self, field, species: str, component: str, prec: str = "f64"):
        """a compact n^3 field: a numpy array (host) or a device pointer (int)"""
        if isinstance(field, np.ndarray):
            dt = np.float64 if field.dtype == np.float64 else np.float32
            a = np.ascontiguousarray(field, dtype=dt)
            rc = lib().mf_grafic2_write_field(self.ptr, a.ctypes.data,
                                              L.MF_PREC_F64 if dt == np.float64 else L.MF_PREC_F32, L.MF_LOC_HOST,
                                              SPECIES[species], COMPONENTS[component])
        else:
            rc = lib().mf_grafic2_write_field(self.ptr, C.c_void_p(int(field)),
                                              L.MF_PREC_F64 if prec == "f64" else L.MF_PREC_F32, L.MF_LOC_DEVICE,
                                              SPECIES[species], COMPONENTS[component])
        _check(self.ctx.ptr, rc)

    def write_ic(self, gen):
        """run an ICGenerator created with out_kind="fields" and the plugin's
        units and write the six dark-matter components"""
        _check(self.ctx.ptr, lib().mf_ic_write_grafic2(gen.ptr, self.ptr))

    def last_write(self) -> dict:
        b, k, w = C.c_size_t(), C.c_double(), C.c_double()
        _check(self.ctx.ptr, lib().mf_grafic2_last_write(self.ptr, C.byref(b), C.byref(k), C.byref(w)))
        return {"bytes": b.value, "kernel_ms": k.value, "wall_ms": w.value}

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_grafic2_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
