"""ctypes bindings of include/snow_mpm.h (the library's C ABI).

Loading fails loudly when the CUDA library is missing: there is no CPU
fallback in the product."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsnow_gb300.so")

(SNOW_OK, SNOW_EINVAL, SNOW_ENOMEM, SNOW_EBUDGET, SNOW_ETIMEDOUT, SNOW_ENUMERIC, SNOW_ECUDA, SNOW_ESTATE,
 SNOW_EUNSUPPORTED, SNOW_ECAPACITY) = (0, -1, -2, -3, -4, -5, -6, -7, -8, -9)
STATUS_NAMES = {0: "SNOW_OK", -1: "SNOW_EINVAL", -2: "SNOW_ENOMEM", -3: "SNOW_EBUDGET", -4: "SNOW_ETIMEDOUT",
                -5: "SNOW_ENUMERIC", -6: "SNOW_ECUDA", -7: "SNOW_ESTATE", -8: "SNOW_EUNSUPPORTED",
                -9: "SNOW_ECAPACITY"}
MODE_REFERENCE, MODE_FAST = 0, 1
(K_RIGID_ADVANCE, K_G_RESET, K_P2G, K_G_FORCE, K_G2P, K_P_ADVANCE, K_G_MASS, K_P_VOLUME) = range(8)

# Every symbol include/snow_mpm.h declares.
EXPORTS = [
    "snow_params_default", "snow_default_walls", "snow_ctx_create", "snow_ctx_destroy", "snow_last_error",
    "snow_ctx_bytes_in_use", "snow_ctx_set_profiling", "snow_ctx_stream", "snow_ctx_synchronize","snow_scene_create",
    "snow_scene_destroy", "snow_scene_footprint", "snow_scene_upload", "snow_scene_upload_std140",
    "snow_scene_set_volume", "snow_scene_init", "snow_scene_step", "snow_dispatch", "snow_scene_download", "snow_scene_download_std140",
    "snow_scene_download_grid", "snow_scene_download_colliders", "snow_scene_stats", "snow_scene_size",
    "snow_scene_cell_keys", "snow_scene_phase_times", "snow_batch_create", "snow_batch_destroy",
    "snow_batch_step", "snow_batch_autotune", "snow_sort_keys_static", "snow_server_create", "snow_server_destroy",
    "snow_server_submit", "snow_server_poll", "snow_server_fetch", "snow_server_stats", "snow_server_drain",
    "snow_scene_set_tuning", "snow_batch_set_tuning", "snow_ctx_set_graphs", "snow_scene_stats_enqueue",
    "snow_ctx_stats_read", "snow_scene_solver_report", "snow_scene_check", "snow_scene_set_wait_limit",
]
SORT_STATIC_MAX_KEYS = 262144  # SNOW_SORT_STATIC_MAX_KEYS


class SnowParams(C.Structure):
    _fields_ = [("grid_pos", C.c_float * 3), ("grid_dim", C.c_int * 3), ("grid_spacing", C.c_float),
                ("young", C.c_float), ("poisson", C.c_float), ("hardening", C.c_float),
                ("crit_compression", C.c_float), ("crit_stretch", C.c_float), ("alpha", C.c_float),
                ("gravity", C.c_float * 3), ("mode", C.c_int), ("sort_interval", C.c_int),
                ("implicit_beta", C.c_float), ("implicit_tolerance", C.c_float), ("implicit_max_iters", C.c_int)]


class SnowCollider(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("type", C.c_int32), ("vel", C.c_float * 3), ("radius", C.c_float),
                ("normal", C.c_float * 3), ("friction", C.c_float)]


class SnowStats(C.Structure):
    _fields_ = [("mass", C.c_double), ("momentum", C.c_double * 3), ("kinetic_energy", C.c_double),
                ("center_of_mass", C.c_double * 3), ("bbox_min", C.c_double * 3), ("bbox_max", C.c_double * 3),
                ("mean_jp", C.c_double), ("nonfinite", C.c_uint64), ("n", C.c_uint64)]


class SnowPhaseTimes(C.Structure):
    _fields_ = [("sort_ms", C.c_double), ("p2g_ms", C.c_double), ("grid_ms", C.c_double), ("g2p_ms", C.c_double),
                ("other_ms", C.c_double), ("total_ms", C.c_double), ("steps", C.c_uint64),
                ("binnings", C.c_uint64), ("wide", C.c_uint64)]


class SnowSolverReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("max_iters", C.c_int), ("residual", C.c_double),
                ("initial_residual", C.c_double)]


class SnowTuning(C.Structure):
    _fields_ = [("sort_interval", C.c_int), ("items_max", C.c_int), ("ctas_per_sm", C.c_int),
                ("steps_taken", C.c_int), ("ms_per_step", C.c_double)]


SERVE_FIFO, SERVE_SRPT = 0, 1


class SnowServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_size_t), ("max_active", C.c_int),
                ("chunk_steps", C.c_int), ("max_active_particles", C.c_size_t), ("policy", C.c_int)]


class SnowJobDesc(C.Structure):
    _fields_ = [("params", C.POINTER(SnowParams)), ("colliders", C.POINTER(SnowCollider)),
                ("n_colliders", C.c_int), ("x", C.POINTER(C.c_float)), ("v", C.POINTER(C.c_float)),
                ("m", C.POINTER(C.c_float)), ("n", C.c_size_t), ("steps", C.c_int), ("dt", C.c_double),
                ("keep_state", C.c_int)]


class SnowJobResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("n", C.c_size_t), ("steps", C.c_int),
                ("queue_s", C.c_double), ("service_s", C.c_double), ("latency_s", C.c_double),
                ("stats", SnowStats)]


class SnowServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("failed", C.c_uint64), ("pending", C.c_uint64), ("active", C.c_uint64),
                ("particle_steps", C.c_double), ("busy_s", C.c_double), ("uptime_s", C.c_double),
                ("resident_bytes", C.c_size_t)]


class SnowError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} missing: build it with snow_gb300.build.build() (needs nvcc)")
    L = C.CDLL(path)
    vp, fp, ip, up, sz = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_uint32), C.c_size_t
    L.snow_params_default.argtypes = [C.POINTER(SnowParams)]
    L.snow_params_default.restype = None
    L.snow_default_walls.argtypes = [C.POINTER(SnowParams), C.POINTER(SnowCollider)]
    L.snow_ctx_create.argtypes = [C.c_int, sz, C.POINTER(vp)]
    L.snow_ctx_destroy.argtypes = [vp]
    L.snow_ctx_destroy.restype = None
    L.snow_last_error.argtypes = [vp]
    L.snow_last_error.restype = C.c_char_p
    L.snow_ctx_bytes_in_use.argtypes = [vp]
    L.snow_ctx_bytes_in_use.restype = sz
    L.snow_ctx_set_profiling.argtypes = [vp, C.c_int]
    L.snow_ctx_set_graphs.argtypes = [vp, C.c_int]
    L.snow_ctx_synchronize.argtypes = [vp]
    L.snow_ctx_stream.argtypes = [vp]
    L.snow_ctx_stream.restype = vp
    L.snow_scene_create.argtypes = [vp, C.POINTER(SnowParams), C.POINTER(SnowCollider), C.c_int, sz, C.POINTER(vp)]
    L.snow_scene_destroy.argtypes = [vp]
    L.snow_scene_destroy.restype = None
    L.snow_scene_footprint.argtypes = [C.POINTER(SnowParams), sz]
    L.snow_scene_footprint.restype = sz
    L.snow_scene_upload.argtypes = [vp, fp, fp, fp, fp, fp, sz]
    L.snow_scene_upload_std140.argtypes = [vp, fp, ip, fp, fp, sz]
    L.snow_scene_set_volume.argtypes = [vp, fp, sz]
    L.snow_scene_init.argtypes = [vp]
    L.snow_scene_step.argtypes = [vp, C.c_double, C.c_int]
    L.snow_dispatch.argtypes = [vp, C.c_int, C.c_double]
    L.snow_scene_download.argtypes = [vp, fp, fp, fp, fp, fp, fp]
    L.snow_scene_download_std140.argtypes = [vp, fp, ip, fp, fp]
    L.snow_scene_download_grid.argtypes = [vp, fp, fp, fp, fp]
    L.snow_scene_download_colliders.argtypes = [vp, C.POINTER(SnowCollider)]
    L.snow_scene_stats.argtypes = [vp, C.POINTER(SnowStats)]
    L.snow_scene_stats_enqueue.argtypes = [vp, C.c_int]
    L.snow_ctx_stats_read.argtypes = [vp, C.c_int, C.POINTER(SnowStats)]
    L.snow_scene_size.argtypes = [vp]
    L.snow_scene_size.restype = sz
    L.snow_scene_cell_keys.argtypes = [vp, up, up]
    L.snow_scene_phase_times.argtypes = [vp, C.POINTER(SnowPhaseTimes), C.c_int]
    L.snow_scene_solver_report.argtypes = [vp, C.POINTER(SnowSolverReport)]
    L.snow_batch_create.argtypes = [vp, C.POINTER(vp), C.c_int, C.POINTER(vp)]
    L.snow_batch_destroy.argtypes = [vp]
    L.snow_batch_destroy.restype = None
    L.snow_batch_step.argtypes = [vp, C.POINTER(C.c_double), C.c_int]
    L.snow_batch_autotune.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(SnowTuning)]
    L.snow_batch_set_tuning.argtypes = [vp, C.POINTER(SnowTuning)]
    L.snow_scene_set_tuning.argtypes = [vp, C.POINTER(SnowTuning)]
    L.snow_sort_keys_static.argtypes = [vp, vp, vp, sz, C.c_int, vp]
    L.snow_scene_check.argtypes = [vp]
    L.snow_scene_set_wait_limit.argtypes = [vp, C.c_uint32, C.c_uint32]
    L.snow_server_create.argtypes = [C.POINTER(SnowServerConfig), C.POINTER(vp)]
    L.snow_server_destroy.argtypes = [vp]
    L.snow_server_destroy.restype = None
    L.snow_server_submit.argtypes = [vp, C.POINTER(SnowJobDesc), C.POINTER(C.c_uint64)]
    L.snow_server_poll.argtypes = [vp, C.POINTER(SnowJobResult), C.c_int, C.POINTER(C.c_int)]
    L.snow_server_fetch.argtypes = [vp, C.c_uint64, fp, fp, fp, fp]
    L.snow_server_stats.argtypes = [vp, C.POINTER(SnowServerStats)]
    L.snow_server_drain.argtypes = [vp, C.c_double]
    _lib = L
    return L


def ptr(a, t=C.c_float):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))
