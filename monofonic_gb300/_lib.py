"""ctypes binding of libmfgpu (the C ABI declared in include/monofonic_gb300.h).

The library is loaded from the package directory.  There is no fallback: if
the shared object is missing or fails to load, importing raises, so nothing
silently runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmfgpu.so")

MF_OK, MF_ERR_ARG, MF_ERR_SHAPE, MF_ERR_OOM, MF_ERR_CUDA, MF_ERR_TIMEOUT, MF_ERR_CANCELLED, MF_ERR_STATE, MF_ERR_IO = range(9)
MF_PREC_F64, MF_PREC_F32 = 0, 1
MF_SPACE_R, MF_SPACE_K = 0, 1
MF_CONV_ORSZAG, MF_CONV_NAIVE = 0, 1
MF_OPND_PLAIN, MF_OPND_HESS, MF_OPND_SUM, MF_OPND_DIFF, MF_OPND_GRAD = range(5)
MF_OP_ASSIGN, MF_OP_ADD, MF_OP_SUB, MF_OP_AXPY = range(4)

ERROR_NAMES = {1: "MF_ERR_ARG", 2: "MF_ERR_SHAPE", 3: "MF_ERR_OOM", 4: "MF_ERR_CUDA",
               5: "MF_ERR_TIMEOUT", 6: "MF_ERR_CANCELLED", 7: "MF_ERR_STATE",
               8: "MF_ERR_IO"}


class mf_operand(C.Structure):
    _fields_ = [("grid", C.c_void_p), ("kind", C.c_int), ("d", C.c_int * 4)]


# name -> (restype, argtypes); every C-ABI symbol the header declares
SIGNATURES = {
    "mf_version": (C.c_char_p, []),
    "mf_ctx_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "mf_ctx_launch_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "mf_ctx_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "mf_ctx_profile_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mf_probe_fma_rate": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "mf_selftest_bounded_wait": (C.c_int, [C.c_void_p, C.c_long]),
    "mf_selftest_float_pairs": (C.c_int, [C.c_void_p, C.c_longlong, C.c_uint64, C.c_double, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_longlong)]),
    "mf_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "mf_host_free": (C.c_int, [C.c_void_p]),
    "mf_host_huge_page_bytes": (C.c_int, [C.POINTER(C.c_size_t)]),
    "mf_grid_size_supported": (C.c_int, [C.c_int]),
    "mf_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "mf_ctx_destroy": (C.c_int, [C.c_void_p]),
    "mf_last_error": (C.c_char_p, [C.c_void_p]),
    "mf_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "mf_grid_create": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "mf_grid_destroy": (C.c_int, [C.c_void_p]),
    "mf_grid_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                               C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]),
    "mf_grid_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "mf_grid_download": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mf_grid_fill_real64": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mf_grid_fft_forward": (C.c_int, [C.c_void_p, C.c_int]),
    "mf_grid_fft_backward": (C.c_int, [C.c_void_p, C.c_int]),
    "mf_grid_zero": (C.c_int, [C.c_void_p]),
    "mf_grid_scale": (C.c_int, [C.c_void_p, C.c_double]),
    "mf_grid_zero_dc": (C.c_int, [C.c_void_p]),
    "mf_grid_inverse_laplacian": (C.c_int, [C.c_void_p]),
    "mf_grid_shift": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int]),
    "mf_cgrid_fft": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "mf_grid_write_power_spectrum": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mf_grid_power_spectrum": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                         C.POINTER(C.c_int)]),
    "mf_conv_create": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "mf_conv_destroy": (C.c_int, [C.c_void_p]),
    "mf_conv_convolve2": (C.c_int, [C.c_void_p, C.POINTER(mf_operand), C.POINTER(mf_operand), C.c_void_p,
                                    C.c_int, C.c_double]),
    "mf_conv_convolve2_invlap": (C.c_int, [C.c_void_p, C.POINTER(mf_operand), C.POINTER(mf_operand), C.c_void_p,
                                           C.c_int, C.c_double]),
    "mf_conv_convolve3": (C.c_int, [C.c_void_p, C.POINTER(mf_operand), C.POINTER(mf_operand),
                                    C.POINTER(mf_operand), C.c_void_p, C.c_int, C.c_double]),
}


class mf_cosmo_params(C.Structure):
    _fields_ = [("Omega_m", C.c_double), ("Omega_b", C.c_double), ("h", C.c_double), ("sigma_8", C.c_double),
                ("n_s", C.c_double), ("Omega_L", C.c_double), ("Tcmb", C.c_double), ("m_nu1", C.c_double),
                ("N_ur", C.c_double), ("w_0", C.c_double), ("w_a", C.c_double), ("zero_radiation", C.c_int)]


class mf_cosmo_scalars(C.Structure):
    _fields_ = [("Dplus", C.c_double), ("vfac", C.c_double), ("f", C.c_double), ("pnorm", C.c_double),
                ("sigma8_measured", C.c_double), ("n_s", C.c_double), ("h", C.c_double), ("H0", C.c_double),
                ("Omega_m", C.c_double), ("Omega_b", C.c_double), ("Omega_r", C.c_double),
                ("Omega_DE", C.c_double), ("Tcmb", C.c_double)]


class mf_ic_params(C.Structure):
    _fields_ = [("ngrid", C.c_int), ("boxlen", C.c_double), ("zstart", C.c_double), ("lpt_order", C.c_int),
                ("lattice", C.c_int), ("precision", C.c_int), ("convolver", C.c_int), ("fixing", C.c_int),
                ("inversion", C.c_int), ("plt", C.c_int), ("cosmo", mf_cosmo_scalars),
                ("tk_table", C.c_void_p), ("lunit", C.c_double), ("vunit", C.c_double), ("out_kind", C.c_int),
                ("pos64", C.c_int), ("id64", C.c_int), ("plt_ngrid", C.c_int),
                ("per_term_conv", C.c_int), ("baryons", C.c_int), ("baryon_vrel", C.c_int), ("munit", C.c_double),
                ("tk_dbc_table", C.c_void_p), ("tk_tbc_table", C.c_void_p), ("Dplus_target", C.c_double)]


class mf_particles(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("ids", C.c_void_p), ("npart", C.c_int64),
                ("location", C.c_int), ("mass", C.c_void_p)]


MF_OUT_PARTICLES, MF_OUT_FIELDS = 0, 1
MF_LOC_HOST, MF_LOC_DEVICE = 0, 1

SIGNATURES.update({
    "mf_cosmo_params_default": (None, [C.POINTER(mf_cosmo_params)]),
    "mf_cosmology_compute": (C.c_int, [C.POINTER(mf_cosmo_params), C.c_double, C.POINTER(mf_cosmo_scalars)]),
    "mf_eh_transfer": (C.c_int, [C.POINTER(mf_cosmo_params), C.c_void_p, C.c_void_p, C.c_size_t]),
    "mf_white_noise_host": (C.c_int, [C.c_int, C.c_uint64, C.c_void_p, C.c_int]),
    "mf_ic_output_size": (C.c_int, [C.POINTER(mf_ic_params), C.POINTER(C.c_int64), C.POINTER(C.c_size_t),
                                    C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "mf_ic_device_footprint": (C.c_int, [C.POINTER(mf_ic_params), C.POINTER(C.c_size_t)]),
    "mf_ic_create": (C.c_int, [C.c_void_p, C.POINTER(mf_ic_params), C.POINTER(C.c_void_p)]),
    "mf_ic_destroy": (C.c_int, [C.c_void_p]),
    "mf_ic_set_noise": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "mf_ic_run": (C.c_int, [C.c_void_p, C.POINTER(mf_particles)]),
    "mf_ic_run_async": (C.c_int, [C.c_void_p, C.POINTER(mf_particles)]),
    "mf_ic_wait": (C.c_int, [C.c_void_p]),
    "mf_ic_stage_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "mf_ic_get_potential": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "mf_ic_get_noise": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "mf_plt_tables": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mf_grid_fill_white_noise": (C.c_int, [C.c_void_p, C.c_uint64]),
    "mf_copy_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "mf_ic_set_noise_seed": (C.c_int, [C.c_void_p, C.c_uint64]),
    "mf_ic_set_cosmology": (C.c_int, [C.c_void_p, C.POINTER(mf_cosmo_scalars)]),
    "mf_ic_enqueue": (C.c_int, [C.c_void_p]),
    "mf_ic_particles": (C.c_int, [C.c_void_p, C.POINTER(mf_particles)]),
    "mf_ic_run_species": (C.c_int, [C.c_void_p, C.POINTER(mf_particles), C.c_int]),
    "mf_ic_particles_species": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(mf_particles)]),
    "mf_ic_mass_bytes": (C.c_int, [C.POINTER(mf_ic_params), C.POINTER(C.c_size_t)]),
    "mf_ic_context": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
})


class mf_ic_request(C.Structure):
    _fields_ = [("ngrid", C.c_int), ("boxlen", C.c_double), ("zstart", C.c_double), ("lpt_order", C.c_int),
                ("lattice", C.c_int), ("precision", C.c_int), ("cosmo", mf_cosmo_params), ("seed", C.c_uint64),
                ("pos64", C.c_int), ("id64", C.c_int)]


MF_OUTPUT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int64, C.POINTER(mf_particles), C.c_int64, C.c_int64, C.c_int)


class mf_server_config(C.Structure):
    _fields_ = [("nworkers", C.c_int), ("hbm_budget", C.c_size_t), ("chunk_particles", C.c_int64),
                ("output", MF_OUTPUT_FN), ("user", C.c_void_p), ("starvation_s", C.c_double)]


class mf_request_result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("npart", C.c_int64), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_gpu_done", C.c_double), ("t_done", C.c_double), ("gpu_ms", C.c_double)]


class mf_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("running", C.c_int64), ("bytes_in_use", C.c_size_t), ("bytes_budget", C.c_size_t),
                ("peak_bytes", C.c_size_t), ("pooled_pipelines", C.c_int), ("t_now", C.c_double)]


SIGNATURES.update({
    "mf_batch_create": (C.c_int, [C.c_int, C.POINTER(mf_ic_request), C.c_int, C.c_int, C.c_int,
                                  C.POINTER(C.c_void_p)]),
    "mf_batch_tuning": (C.c_char_p, [C.c_void_p]),
    "mf_autotune": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_size_t]),
    "mf_autotune_reset": (C.c_int, []),
    "mf_schedule_set": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "mf_batch_destroy": (C.c_int, [C.c_void_p]),
    "mf_batch_set_items": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(mf_cosmo_params),
                                     C.POINTER(C.c_uint64), C.c_int]),
    "mf_batch_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "mf_batch_particles": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(mf_particles)]),
    "mf_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_size_t)]),
    "mf_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "mf_server_create": (C.c_int, [C.c_int, C.POINTER(mf_server_config), C.POINTER(C.c_void_p)]),
    "mf_server_submit": (C.c_int, [C.c_void_p, C.POINTER(mf_ic_request), C.POINTER(C.c_int64)]),
    "mf_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(mf_request_result), C.c_double]),
    "mf_server_poll": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(mf_request_result), C.POINTER(C.c_int)]),
    "mf_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "mf_server_release": (C.c_int, [C.c_void_p, C.c_int64]),
    "mf_server_drain": (C.c_int, [C.c_void_p, C.c_double]),
    "mf_server_stats_get": (C.c_int, [C.c_void_p, C.POINTER(mf_server_stats)]),
    "mf_server_now": (C.c_double, [C.c_void_p]),
    "mf_server_last_error": (C.c_char_p, [C.c_void_p]),
    "mf_server_destroy": (C.c_int, [C.c_void_p]),
})



class mf_grafic2_params(C.Structure):
    _fields_ = [("dirname", C.c_char_p), ("ngrid", C.c_int), ("boxlen", C.c_double), ("zstart", C.c_double),
                ("H0", C.c_double), ("Omega_m", C.c_double), ("Omega_DE", C.c_double), ("Omega_b", C.c_double),
                ("baryons", C.c_int), ("ramses_nml", C.c_int), ("use_spt", C.c_int), ("chunk_planes", C.c_int)]


MF_FC_DENSITY, MF_FC_VX, MF_FC_VY, MF_FC_VZ, MF_FC_DX, MF_FC_DY, MF_FC_DZ, MF_FC_MASS = range(8)
MF_SPECIES_DM, MF_SPECIES_BARYON, MF_SPECIES_NEUTRINO = range(3)
MF_OUTTYPE_PARTICLES, MF_OUTTYPE_FIELD_LAGRANGIAN, MF_OUTTYPE_FIELD_EULERIAN = range(3)

SIGNATURES.update({
    "mf_grafic2_create": (C.c_int, [C.c_void_p, C.POINTER(mf_grafic2_params), C.POINTER(C.c_void_p)]),
    "mf_grafic2_destroy": (C.c_int, [C.c_void_p]),
    "mf_grafic2_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mf_grafic2_write_grid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "mf_grafic2_write_field": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "mf_ic_write_grafic2": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mf_grafic2_last_write": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]),
})

_lib = None


def load():
    """Load libmfgpu.so (raises OSError/ImportError if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libmfgpu.so not built at {LIB_PATH}; run monofonic_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class MFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code
