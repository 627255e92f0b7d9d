"""IC-level API: host cosmology, the white-noise plugin and the LPT pipeline
of ic_generator::run (src/ic_generator.cc:90-948) over libmfgpu's C ABI
(include/monofonic_gb300_ic.h)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import Context, Grid_FFT, lib, _check, MFError

LATTICES = {"sc": 0, "bcc": 1, "fcc": 2, "rsc": 3}


@dataclass
class Cosmology:
    """[cosmology] section, ParameterSet = none (cosmology_parameters.hh:84-150)."""
    Omega_m: float = 0.3099
    Omega_b: float = 0.0488
    h: float = 0.6774
    sigma_8: float = 0.8102
    n_s: float = 0.9667
    Omega_L: float = -1.0
    Tcmb: float = -1.0
    m_nu1: float = -1.0
    N_ur: float = -1.0
    w_0: float = -1.0
    w_a: float = 0.0
    zero_radiation: bool = False

    def to_c(self):
        p = L.mf_cosmo_params()
        for f in ("Omega_m", "Omega_b", "h", "sigma_8", "n_s", "Omega_L", "Tcmb", "m_nu1", "N_ur", "w_0", "w_a"):
            setattr(p, f, float(getattr(self, f)))
        p.zero_radiation = int(self.zero_radiation)
        return p


def cosmology_scalars(cosmo: Cosmology, zstart: float):
    """cosmology::calculator scalars at z_start (D+, vfac, pnorm, ...)."""
    out = L.mf_cosmo_scalars()
    rc = lib().mf_cosmology_compute(C.byref(cosmo.to_c()), float(zstart), C.byref(out))
    if rc != L.MF_OK:
        raise MFError(rc, "mf_cosmology_compute")
    return out


def eh_transfer(cosmo: Cosmology, k):
    k = np.ascontiguousarray(k, dtype=np.float64)
    out = np.empty_like(k)
    rc = lib().mf_eh_transfer(C.byref(cosmo.to_c()), k.ctypes.data, out.ctypes.data, k.size)
    if rc != L.MF_OK:
        raise MFError(rc, "mf_eh_transfer")
    return out


def white_noise(n: int, seed: int, nthreads: int = 0) -> np.ndarray:
    """Project RNG plugin: n^3 float64 N(0,1) noise (Philox4x32-10 + Box-Muller)."""
    out = np.empty((n, n, n), dtype=np.float64)
    rc = lib().mf_white_noise_host(int(n), C.c_uint64(seed), out.ctypes.data, int(nthreads))
    if rc != L.MF_OK:
        raise MFError(rc, "mf_white_noise_host")
    return out


@dataclass
class ICConfig:
    """[setup] keys of the path (ic_generator.cc:98-149) plus output options."""
    ngrid: int
    boxlen: float
    zstart: float
    lpt_order: int = 3
    lattice: str = "sc"
    precision: str = "f64"
    convolver: str = "orszag"
    fixing: bool = False
    inversion: bool = False
    plt: bool = False
    lunit: float = 1.0
    vunit: float = 1.0
    out_kind: str = "particles"
    pos64: bool = True
    id64: bool = True
    plt_ngrid: int = 0
    per_term_conv: bool = False
    baryons: bool = False       # setup/DoBaryons: dark matter + baryon particles with masses
    baryon_vrel: bool = False   # setup/DoBaryonVrel
    munit: float = 1.0          # output_plugin::mass_unit
    Dplus_target: float = 0.0   # D+ at ztarget (0: 1)

    def to_c(self, scalars, tk_table=None, tk_dbc=None, tk_tbc=None):
        p = L.mf_ic_params()
        p.ngrid = self.ngrid
        p.boxlen = self.boxlen
        p.zstart = self.zstart
        p.lpt_order = self.lpt_order
        p.lattice = LATTICES[self.lattice]
        p.precision = L.MF_PREC_F64 if self.precision == "f64" else L.MF_PREC_F32
        p.convolver = L.MF_CONV_ORSZAG if self.convolver == "orszag" else L.MF_CONV_NAIVE
        p.fixing = int(self.fixing)
        p.inversion = int(self.inversion)
        p.plt = int(self.plt)
        p.cosmo = scalars
        p.tk_table = tk_table.ctypes.data if tk_table is not None else None
        p.lunit = self.lunit
        p.vunit = self.vunit
        p.out_kind = L.MF_OUT_PARTICLES if self.out_kind == "particles" else L.MF_OUT_FIELDS
        p.pos64 = int(self.pos64)
        p.id64 = int(self.id64)
        p.plt_ngrid = int(self.plt_ngrid)
        p.per_term_conv = int(self.per_term_conv)
        p.baryons = int(self.baryons)
        p.baryon_vrel = int(self.baryon_vrel)
        p.munit = float(self.munit)
        p.tk_dbc_table = tk_dbc.ctypes.data if tk_dbc is not None else None
        p.tk_tbc_table = tk_tbc.ctypes.data if tk_tbc is not None else None
        p.Dplus_target = float(self.Dplus_target)
        return p


class ICGenerator:
    """Device-resident LPT pipeline for one parameter set."""

    def __init__(self, ctx: Context, cfg: ICConfig, scalars, tk_table=None, tk_dbc=None, tk_tbc=None):
        """tk_table, tk_dbc, tk_tbc: optional host tables of T_delta_matter,
        T_delta_bc and T_theta_bc at k = sqrt(k2)*2pi/L, k2 = 0..3(n/2)^2"""
        self.ctx, self.cfg = ctx, cfg
        as64 = lambda t: None if t is None else np.ascontiguousarray(t, dtype=np.float64)
        self._tk, self._tdbc, self._ttbc = as64(tk_table), as64(tk_dbc), as64(tk_tbc)
        self.params = cfg.to_c(scalars, self._tk, self._tdbc, self._ttbc)
        p = C.c_void_p()
        _check(ctx.ptr, lib().mf_ic_create(ctx.ptr, C.byref(self.params), C.byref(p)))
        self.ptr = p
        np_, pb, vb, ib = C.c_int64(), C.c_size_t(), C.c_size_t(), C.c_size_t()
        lib().mf_ic_output_size(C.byref(self.params), C.byref(np_), C.byref(pb), C.byref(vb), C.byref(ib))
        self.npart, self.pos_bytes, self.vel_bytes, self.id_bytes = np_.value, pb.value, vb.value, ib.value

    def set_noise(self, noise: np.ndarray):
        a = np.ascontiguousarray(noise, dtype=np.float64)
        _check(self.ctx.ptr, lib().mf_ic_set_noise(self.ptr, a.ctypes.data, L.MF_LOC_HOST))

    def set_noise_device(self, dptr: int):
        _check(self.ctx.ptr, lib().mf_ic_set_noise(self.ptr, C.c_void_p(dptr), L.MF_LOC_DEVICE))

    def set_noise_seed(self, seed: int):
        """white noise of the project RNG plugin generated on the device at
        the start of every run (the same bits as white_noise(n, seed))"""
        _check(self.ctx.ptr, lib().mf_ic_set_noise_seed(self.ptr, C.c_uint64(int(seed))))

    def set_cosmology(self, scalars):
        """new cosmology scalars (cosmology_scalars) for the next run"""
        _check(self.ctx.ptr, lib().mf_ic_set_cosmology(self.ptr, C.byref(scalars)))
        self.params.cosmo = scalars

    def set_noise_host_ptr(self, hptr: int):
        """noise from a host pointer (e.g. page-locked memory of mf_host_alloc)."""
        _check(self.ctx.ptr, lib().mf_ic_set_noise(self.ptr, C.c_void_p(hptr), L.MF_LOC_HOST))

    def run_into(self, pos_ptr: int, vel_ptr: int, ids_ptr: int):
        """run and copy the particles into caller-owned host buffers."""
        out = L.mf_particles()
        out.pos, out.vel, out.ids = pos_ptr, vel_ptr, ids_ptr
        out.location = L.MF_LOC_HOST
        _check(self.ctx.ptr, lib().mf_ic_run(self.ptr, C.byref(out)))

    def run_into_async(self, pos_ptr: int, vel_ptr: int, ids_ptr: int):
        """queue a run whose particles are copied into caller-owned host
        buffers (page-locked for overlap) and return at once; the buffers are
        complete after wait().  The next queued run computes while this one's
        particles are still being copied."""
        out = L.mf_particles()
        out.pos, out.vel, out.ids = pos_ptr, vel_ptr, ids_ptr
        out.location = L.MF_LOC_HOST
        _check(self.ctx.ptr, lib().mf_ic_run_async(self.ptr, C.byref(out)))

    def wait(self):
        """wait for every queued run, host copies included"""
        _check(self.ctx.ptr, lib().mf_ic_wait(self.ptr))

    def run(self, to_host: bool = True):
        """Run the pipeline; returns (pos, vel, ids) numpy arrays, or device
        pointers when to_host is False."""
        cfg = self.cfg
        out = L.mf_particles()
        if to_host:
            if cfg.out_kind == "fields":
                pos = np.empty((3, cfg.ngrid, cfg.ngrid, cfg.ngrid))
                vel = np.empty_like(pos)
                ids = None
            else:
                rt = np.float64 if cfg.pos64 else np.float32
                pos = np.empty((self.npart, 3), dtype=rt)
                vel = np.empty((self.npart, 3), dtype=rt)
                ids = np.empty(self.npart, dtype=np.uint64 if cfg.id64 else np.uint32)
            out.pos, out.vel = pos.ctypes.data, vel.ctypes.data
            out.ids = ids.ctypes.data if ids is not None else None
            out.location = L.MF_LOC_HOST
            _check(self.ctx.ptr, lib().mf_ic_run(self.ptr, C.byref(out)))
            return pos, vel, ids
        out.location = L.MF_LOC_DEVICE
        _check(self.ctx.ptr, lib().mf_ic_run(self.ptr, C.byref(out)))
        return out.pos, out.vel, out.ids

    def run_species(self, to_host: bool = True):
        """two-species run (cfg.baryons): {"dm": (pos, vel, ids, mass),
        "baryon": (...)} as numpy arrays, or device pointers.  With field
        output: dm = (displacements [3,n,n,n], velocities, None, mass field
        [n,n,n]) and baryon = (density contrast [n,n,n], Eulerian velocities
        [3,n,n,n], None, None) from the semiclassical branch."""
        outs = (L.mf_particles * 2)()
        keep = []
        if to_host:
            cfg = self.cfg
            n = cfg.ngrid
            for sp in range(2):
                if cfg.out_kind == "fields":
                    # dark matter: dx,dy,dz / vx,vy,vz grids and the mass field;
                    # baryons (Eulerian branch): density contrast and vx,vy,vz
                    arrs = ((np.empty((3, n, n, n)) if sp == 0 else np.empty((n, n, n))), np.empty((3, n, n, n)),
                            None, np.empty((n, n, n)) if sp == 0 else None)
                else:
                    rt = np.float64 if cfg.pos64 else np.float32
                    arrs = (np.empty((self.npart, 3), dtype=rt), np.empty((self.npart, 3), dtype=rt),
                            np.empty(self.npart, dtype=np.uint64 if cfg.id64 else np.uint32),
                            np.empty(self.npart, dtype=rt))
                keep.append(arrs)
                outs[sp].pos, outs[sp].vel, outs[sp].ids, outs[sp].mass = (
                    a.ctypes.data if a is not None else None for a in arrs)
                outs[sp].location = L.MF_LOC_HOST
        else:
            for sp in range(2):
                outs[sp].location = L.MF_LOC_DEVICE
        _check(self.ctx.ptr, lib().mf_ic_run_species(self.ptr, outs, 2))
        if to_host:
            return {"dm": keep[0], "baryon": keep[1]}
        return {k: (outs[i].pos, outs[i].vel, outs[i].ids, outs[i].mass) for i, k in enumerate(("dm", "baryon"))}

    def stage_times(self):
        ms = (C.c_double * 8)()
        lib().mf_ic_stage_times(self.ptr, ms)
        return list(ms)

    def potential(self, which: int) -> np.ndarray:
        """k-space potential (unscaled) of the last run: 0 phi, 1 phi2, 2 phi3, 3-5 A3."""
        g = C.c_void_p()
        _check(self.ctx.ptr, lib().mf_ic_get_potential(self.ptr, int(which), C.byref(g)))
        n = self.cfg.ngrid
        dt = np.float64 if self.cfg.precision == "f64" else np.float32
        a = np.empty((n, n, n + 2), dtype=dt)
        _check(self.ctx.ptr, lib().mf_grid_download(g, a.ctypes.data))
        return a.view(np.complex128 if dt == np.float64 else np.complex64).reshape(n, n, n // 2 + 1)

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_ic_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host buffer (mf_host_alloc)."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        rc = lib().mf_host_alloc(C.c_size_t(int(nbytes)), C.byref(p))
        if rc != L.MF_OK:
            raise MFError(rc, f"mf_host_alloc({nbytes})")
        self.ptr, self.nbytes = p.value, int(nbytes)

    def array(self, dtype, shape):
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def close(self):
        if getattr(self, "ptr", None):
            lib().mf_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plt_tables(ctx: Context, lattice: str, ng: int = 64):
    """PLT tables (D_r, D_theta, D_phi, vfac correction), each (ng, ng, ng/2+1)."""
    shape = (ng, ng, ng // 2 + 1)
    out = [np.empty(shape) for _ in range(4)]
    _check(ctx.ptr, lib().mf_plt_tables(ctx.ptr, LATTICES[lattice], int(ng), *[a.ctypes.data for a in out]))
    return out


def device_footprint(cfg: ICConfig, scalars) -> int:
    b = C.c_size_t()
    p = cfg.to_c(scalars)
    rc = lib().mf_ic_device_footprint(C.byref(p), C.byref(b))
    if rc != L.MF_OK:
        raise MFError(rc, "mf_ic_device_footprint")
    return b.value


def autotune(ctx: Context, n: int, precision: str = "f32") -> str:
    """mf_autotune: pick the fastest schedule of each convolution pass for grid
    size n (process-wide, used by every later launch); returns the report"""
    buf = C.create_string_buffer(8192)
    prec = L.MF_PREC_F64 if precision == "f64" else L.MF_PREC_F32
    _check(ctx.ptr, lib().mf_autotune(ctx.ptr, int(n), prec, buf, len(buf)))
    return buf.value.decode()


def autotune_reset():
    lib().mf_autotune_reset()
