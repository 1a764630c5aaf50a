"""ctypes binding of libnyxpm.so (include/nyxpm.h).

The library is built in-tree by nyx_gb300/build.py.  There is no fallback: if
the shared library is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnyxpm.so")

NYXPM_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "NOT_CONVERGED",
                5: "TIMEOUT", 6: "NO_DEVICE"}
NYXPM_FP64 = 0
NYXPM_MIXED = 1
NYXPM_STEP_REUSE_FIELD = 1
NUM_STAGES = 12
STAGE_NAMES = ["keys", "scan", "scatter", "gather", "deposit", "rhs", "smooth", "restrict",
               "prolong", "bottom", "norm", "kick"]

# every symbol include/nyxpm.h declares
EXPORTS = [
    "nyxpm_default_params", "nyxpm_create", "nyxpm_destroy", "nyxpm_last_error",
    "nyxpm_abi_version", "nyxpm_stream", "nyxpm_synchronize", "nyxpm_box_create",
    "nyxpm_box_destroy", "nyxpm_box_bytes", "nyxpm_box_upload", "nyxpm_box_download",
    "nyxpm_set_mass_offset", "nyxpm_redistribute", "nyxpm_deposit", "nyxpm_solve_phi",
    "nyxpm_get_phi", "nyxpm_set_phi", "nyxpm_grav_vector", "nyxpm_set_grav_vector",
    "nyxpm_kick_drift", "nyxpm_kick",
    "nyxpm_step", "nyxpm_step_host", "nyxpm_init_field", "nyxpm_integrate_a", "nyxpm_dt_for_da",
    "nyxpm_set_profiling", "nyxpm_get_profile", "nyxpm_launch_count", "nyxpm_measure_fp64_peak",
    "nyxpm_ensemble_create", "nyxpm_ensemble_destroy", "nyxpm_ensemble_box_bytes",
    "nyxpm_ensemble_arena_used", "nyxpm_ensemble_add", "nyxpm_ensemble_remove",
    "nyxpm_ensemble_upload", "nyxpm_ensemble_download", "nyxpm_ensemble_get_phi",
    "nyxpm_ensemble_grav_vector", "nyxpm_ensemble_set_tuning", "nyxpm_ensemble_get_tuning",
    "nyxpm_ensemble_step", "nyxpm_deposit_noalloc",
    "nyxpm_default_dt_params", "nyxpm_est_time_step", "nyxpm_comoving_est_dt",
    "nyxpm_compute_new_dt", "nyxpm_particle_file_count", "nyxpm_particle_file_read",
    "nyxpm_particle_file_write", "nyxpm_write_comoving_a", "nyxpm_read_comoving_a",
    "nyxpm_cosmo_1ppc_particles", "nyxpm_cosmo_ic_factors", "nyxpm_box_init_cosmo_1ppc",
    "nyxpm_multifab_info_read", "nyxpm_multifab_boxes", "nyxpm_multifab_read",
    "nyxpm_multifab_write", "nyxpm_particles_info", "nyxpm_particles_read", "nyxpm_particles_write",
    "nyxpm_amr_create", "nyxpm_amr_destroy", "nyxpm_amr_upload", "nyxpm_amr_download",
    "nyxpm_amr_step", "nyxpm_amr_assign", "nyxpm_amr_deposit", "nyxpm_amr_solve",
    "nyxpm_amr_grav_vector", "nyxpm_amr_kick", "nyxpm_amr_field", "nyxpm_amr_cells",
]
NYXPM_MF_REJECT_NAN = 1


class MultiFabInfo(C.Structure):
    _fields_ = [
        ("ncomp", C.c_int),
        ("ngrow", C.c_int),
        ("nboxes", C.c_int),
        ("lo", C.c_int * 3),
        ("hi", C.c_int * 3),
        ("has_minmax", C.c_int),
    ]
NYXPM_FILE_ASCII, NYXPM_FILE_BINARY, NYXPM_FILE_BINARY_META, NYXPM_FILE_BINARY_F64 = 0, 1, 2, 3


class ParticleHeader(C.Structure):
    _fields_ = [
        ("single_precision", C.c_int),
        ("dim", C.c_int),
        ("n_real_extra", C.c_int),
        ("n_int_extra", C.c_int),
        ("is_checkpoint", C.c_int),
        ("finest_level", C.c_int),
        ("num_particles", C.c_int64),
        ("max_next_id", C.c_int64),
        ("ngrids", C.c_int),
        ("pad", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class Params(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("stream", C.c_void_p),
        ("comoving_OmM", C.c_double),
        ("comoving_OmR", C.c_double),
        ("comoving_h", C.c_double),
        ("gconst", C.c_double),
        ("rel_tol", C.c_double),
        ("max_vcycles", C.c_int),
        ("nu1", C.c_int),
        ("nu2", C.c_int),
        ("verbose", C.c_int),
        ("mixed_inner_vcycles", C.c_int),
        ("mg_fused_edge", C.c_int),
    ]


class DtParams(C.Structure):
    _fields_ = [
        ("cfl", C.c_double),
        ("change_max", C.c_double),
        ("relative_max_change_a", C.c_double),
        ("absolute_max_change_a", C.c_double),
        ("final_a", C.c_double),
        ("stop_time", C.c_double),
        ("dt_binpow", C.c_double),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("vcycles", C.c_int),
        ("inner_vcycles", C.c_int),
        ("resnorm0", C.c_double),
        ("resnorm", C.c_double),
        ("bnorm", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepInfo(C.Structure):
    _fields_ = [("old_solve", SolveInfo), ("new_solve", SolveInfo)]


class Profile(C.Structure):
    _fields_ = [
        ("launches", C.c_int64 * NUM_STAGES),
        ("ms", C.c_double * NUM_STAGES),
        ("bytes", C.c_double * NUM_STAGES),
        ("fine_smooth_launches", C.c_int64),
        ("fine_smooth_ms", C.c_double),
        ("fine_smooth_bytes", C.c_double),
    ]


class Tuning(C.Structure):
    _fields_ = [("deposit_tile", C.c_int), ("smooth_rows", C.c_int), ("inner_vcycles", C.c_int),
                ("max_outer", C.c_int), ("sort_bucket", C.c_int), ("prolong_quad", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class EnsembleInfo(C.Structure):
    _fields_ = [("boxes", C.c_int), ("max_outer_used", C.c_int), ("max_inner_used", C.c_int),
                ("fallback_iters", C.c_int), ("launches", C.c_int), ("pad", C.c_int),
                ("ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


_lib = None


def load(path: str | None = None):
    """Load libnyxpm.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    if path is None:
        if not os.path.exists(LIB_PATH) or _build._stale():
            _build.build()
        path = LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libnyxpm.so not found at {path}; run nyx_gb300/build.py")
    L = C.CDLL(path)
    vp, i64, d = C.c_void_p, C.c_int64, C.c_double
    L.nyxpm_default_params.argtypes = [C.POINTER(Params)]
    L.nyxpm_default_params.restype = None
    L.nyxpm_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.nyxpm_destroy.argtypes = [vp]
    L.nyxpm_destroy.restype = None
    L.nyxpm_last_error.argtypes = [vp]
    L.nyxpm_last_error.restype = C.c_char_p
    L.nyxpm_abi_version.restype = C.c_int
    L.nyxpm_stream.argtypes = [vp]
    L.nyxpm_stream.restype = vp
    L.nyxpm_synchronize.argtypes = [vp]
    L.nyxpm_box_create.argtypes = [vp, C.c_int, d, i64, C.c_int, C.POINTER(vp)]
    L.nyxpm_box_destroy.argtypes = [vp, vp]
    L.nyxpm_box_bytes.argtypes = [C.c_int, i64, C.c_int]
    L.nyxpm_box_bytes.restype = C.c_size_t
    L.nyxpm_box_upload.argtypes = [vp, vp, vp, vp, vp, d]
    L.nyxpm_box_download.argtypes = [vp, vp, vp, vp]
    L.nyxpm_set_mass_offset.argtypes = [vp, vp, C.POINTER(d)]
    L.nyxpm_redistribute.argtypes = [vp, vp]
    L.nyxpm_deposit.argtypes = [vp, vp, vp]
    L.nyxpm_solve_phi.argtypes = [vp, vp, d, C.c_int, C.POINTER(SolveInfo)]
    L.nyxpm_get_phi.argtypes = [vp, vp, vp]
    L.nyxpm_set_phi.argtypes = [vp, vp, vp]
    L.nyxpm_grav_vector.argtypes = [vp, vp, vp]
    L.nyxpm_set_grav_vector.argtypes = [vp, vp, vp, C.c_int]
    L.nyxpm_kick_drift.argtypes = [vp, vp, d, d, d]
    L.nyxpm_kick.argtypes = [vp, vp, d, d, d]
    L.nyxpm_step.argtypes = [vp, vp, d, d, d, C.c_uint, C.POINTER(StepInfo)]
    L.nyxpm_step_host.argtypes = [vp, vp, vp, vp, vp, d, d, d, d, C.c_uint, C.POINTER(StepInfo)]
    L.nyxpm_init_field.argtypes = [vp, vp, d, C.POINTER(SolveInfo)]
    L.nyxpm_integrate_a.argtypes = [C.POINTER(Params), d, d]
    L.nyxpm_integrate_a.restype = d
    L.nyxpm_dt_for_da.argtypes = [C.POINTER(Params), d, d, d]
    L.nyxpm_dt_for_da.restype = d
    L.nyxpm_default_dt_params.argtypes = [C.POINTER(DtParams)]
    L.nyxpm_default_dt_params.restype = None
    L.nyxpm_est_time_step.argtypes = [vp, vp, d, d, C.POINTER(d)]
    L.nyxpm_comoving_est_dt.argtypes = [C.POINTER(Params), d, d, C.POINTER(DtParams), C.POINTER(d)]
    L.nyxpm_compute_new_dt.argtypes = [vp, vp, C.POINTER(DtParams), d, d, d, C.POINTER(d),
                                       C.POINTER(d)]
    cp, sz = C.c_char_p, C.c_size_t
    L.nyxpm_particle_file_count.argtypes = [cp, C.c_int, C.POINTER(i64), cp, sz]
    L.nyxpm_particle_file_read.argtypes = [cp, C.c_int, i64, vp, vp, vp, C.POINTER(i64), cp, sz]
    L.nyxpm_particle_file_write.argtypes = [cp, C.c_int, i64, vp, vp, vp, d, cp, sz]
    L.nyxpm_write_comoving_a.argtypes = [cp, d, cp, sz]
    L.nyxpm_read_comoving_a.argtypes = [cp, C.POINTER(d), cp, sz]
    L.nyxpm_cosmo_1ppc_particles.argtypes = [C.c_int, d, vp, vp, vp, vp, vp, vp]
    L.nyxpm_cosmo_ic_factors.argtypes = [C.POINTER(Params), C.c_int, C.c_int, d, d, vp, vp,
                                         C.POINTER(d)]
    L.nyxpm_box_init_cosmo_1ppc.argtypes = [vp, vp, vp, vp, vp, vp, d]
    L.nyxpm_multifab_info_read.argtypes = [cp, C.POINTER(MultiFabInfo), cp, sz]
    L.nyxpm_multifab_boxes.argtypes = [cp, vp, vp, cp, sz]
    L.nyxpm_multifab_read.argtypes = [cp, C.c_int, C.c_int, vp, vp, C.c_uint, vp, cp, sz]
    L.nyxpm_multifab_write.argtypes = [cp, C.c_int, vp, vp, C.c_int, C.c_int, vp, vp, cp, sz]
    L.nyxpm_particles_info.argtypes = [cp, C.POINTER(ParticleHeader), cp, sz]
    L.nyxpm_particles_read.argtypes = [cp, i64, vp, vp, vp, vp, C.POINTER(i64), cp, sz]
    L.nyxpm_particles_write.argtypes = [cp, C.c_int, i64, vp, vp, vp, d, C.c_int, C.c_int, cp, sz]
    L.nyxpm_set_profiling.argtypes = [vp, C.c_int]
    L.nyxpm_get_profile.argtypes = [vp, C.POINTER(Profile), C.c_int]
    L.nyxpm_launch_count.argtypes = [vp]
    L.nyxpm_launch_count.restype = i64
    L.nyxpm_measure_fp64_peak.argtypes = [vp, C.POINTER(d), C.POINTER(d)]
    dp = C.POINTER(C.c_double)
    L.nyxpm_ensemble_create.argtypes = [vp, C.c_size_t, C.POINTER(vp)]
    L.nyxpm_ensemble_destroy.argtypes = [vp, vp]
    L.nyxpm_ensemble_box_bytes.argtypes = [C.c_int, i64]
    L.nyxpm_ensemble_box_bytes.restype = C.c_size_t
    L.nyxpm_ensemble_arena_used.argtypes = [vp]
    L.nyxpm_ensemble_arena_used.restype = C.c_size_t
    L.nyxpm_ensemble_add.argtypes = [vp, vp, C.c_int, d, i64, C.POINTER(C.c_int)]
    L.nyxpm_ensemble_remove.argtypes = [vp, vp, C.c_int]
    L.nyxpm_ensemble_upload.argtypes = [vp, vp, C.c_int, vp, vp, d]
    L.nyxpm_ensemble_download.argtypes = [vp, vp, C.c_int, vp, vp]
    L.nyxpm_ensemble_get_phi.argtypes = [vp, vp, C.c_int, vp]
    L.nyxpm_ensemble_grav_vector.argtypes = [vp, vp, C.c_int, vp]
    L.nyxpm_ensemble_set_tuning.argtypes = [vp, vp, C.POINTER(Tuning)]
    L.nyxpm_ensemble_get_tuning.argtypes = [vp, vp, C.POINTER(Tuning)]
    L.nyxpm_ensemble_step.argtypes = [vp, vp, dp, dp, dp, C.POINTER(EnsembleInfo)]
    L.nyxpm_deposit_noalloc.argtypes = [vp, vp, vp, i64, d, C.c_int, d, vp, vp, C.c_char_p,
                                        C.c_size_t]
    ip = C.POINTER(C.c_int)
    L.nyxpm_amr_create.argtypes = [vp, C.c_int, d, C.c_int, ip, ip, i64, C.POINTER(vp)]
    L.nyxpm_amr_destroy.argtypes = [vp, vp]
    L.nyxpm_amr_upload.argtypes = [vp, vp, vp, vp, vp, d]
    L.nyxpm_amr_download.argtypes = [vp, vp, vp, vp]
    L.nyxpm_amr_step.argtypes = [vp, vp, d, d, d, C.POINTER(StepInfo)]
    L.nyxpm_amr_assign.argtypes = [vp, vp, vp, vp]
    L.nyxpm_amr_deposit.argtypes = [vp, vp]
    L.nyxpm_amr_solve.argtypes = [vp, vp, d, C.POINTER(SolveInfo)]
    L.nyxpm_amr_grav_vector.argtypes = [vp, vp]
    L.nyxpm_amr_kick.argtypes = [vp, vp, d, d, d, C.c_int]
    L.nyxpm_amr_field.argtypes = [vp, vp, C.c_int, C.c_int, vp]
    L.nyxpm_amr_cells.argtypes = [vp, C.c_int]
    L.nyxpm_amr_cells.restype = i64
    _lib = L
    return L
