"""ctypes binding of libguanaco_gb300.so (the C ABI in include/guanaco_gb300.h).

The library is built in-tree by ``guanaco_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None

GNC_OK = 0
GNC_ERR_INVALID_ARGUMENT = 1
GNC_ERR_UNSUPPORTED = 2
GNC_ERR_CUDA = 3
GNC_ERR_OUT_OF_MEMORY = 4
GNC_ERR_DEVICE = 5
GNC_ERR_PENDING = 6

GNC_STAGE_F32 = 0
GNC_STAGE_F16 = 1
GNC_STAGE_F16T = 2
GNC_INPUT_RAW = 0
GNC_INPUT_CORRECTED = 1

CTF_KIND = {"full": 0, "simple": 1, "simple_real": 2, "simple_imag": 3, "chi": 4, "Es": 5, "Et": 6}

c_size = ctypes.c_size_t
c_float = ctypes.c_float
c_double = ctypes.c_double
c_int = ctypes.c_int
c_void = ctypes.c_void_p


class GncConfig(ctypes.Structure):
    """gnc_config: guanaco::Config (include/guanaco/config.h:29-76)."""

    _fields_ = [
        ("device", c_int),
        ("gpu_index", c_int),
        ("num_pixels", c_size),
        ("num_angles", c_size),
        ("num_defocus", c_size),
        ("grid_height", c_size),
        ("grid_width", c_size),
        ("pixel_size", c_float),
        ("centre", c_float),
        ("min_defocus", c_float),
        ("max_defocus", c_float),
        ("angles", ctypes.POINTER(c_float)),
    ]


class GncCtf(ctypes.Structure):
    """gnc_ctf: guanaco::CTF (include/guanaco/ctf.h:167-178)."""

    _fields_ = [(n, c_double) for n in ("l", "df", "Cs", "Ca", "Pa", "dd", "theta_c", "phi")]


class GncFbpDesc(ctypes.Structure):
    _fields_ = [
        ("num_angles", c_size),
        ("height", c_size),
        ("width", c_size),
        ("grid_height", c_size),
        ("grid_width", c_size),
        ("angles", ctypes.POINTER(c_float)),
        ("centre", ctypes.POINTER(c_float)),
        ("pixel_size", c_float),
        ("input", c_int),
        ("correct", c_int),
        ("num_defocus", c_size),
        ("slab_defocus", ctypes.POINTER(c_double)),
        ("min_defocus", c_float),
        ("max_defocus", c_float),
        ("energy_kev", c_double),
        ("cs_mm", c_double),
        ("astigmatism", c_double),
        ("astigmatism_angle_deg", c_double),
        ("phase_shift_deg", c_double),
        ("weights", ctypes.POINTER(c_double)),
        ("minus", c_int),
        ("staging", c_int),
        ("ctf_pixel_size", c_double),
    ]


class GncRequestInfo(ctypes.Structure):
    """gnc_request_info: outcome and server-clock times of one served request."""

    _fields_ = [("status", c_int), ("graph", c_int), ("device_error", c_int),
                ("t_submit", c_double), ("t_start", c_double), ("t_done", c_double)]


class GncServerStats(ctypes.Structure):
    """gnc_server_stats."""

    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "graph_launches",
                                                "direct_launches", "plans_created",
                                                "plans_evicted")] + \
               [("budget_bytes", c_size), ("bytes_in_use", c_size)] + \
               [(n, c_int) for n in ("slots", "cached_plans", "in_flight", "peak_in_flight",
                                     "queued")]


# Every symbol include/guanaco_gb300.h declares, with (restype, argtypes).
SIGNATURES = {
    "gnc_last_error": (ctypes.c_char_p, []),
    "gnc_version": (c_int, []),
    "gnc_reconstruct": (c_int, [ctypes.POINTER(GncConfig), c_void, c_void]),
    "gnc_reconstruct_device": (c_int, [ctypes.POINTER(GncConfig), c_void, c_void, c_void]),
    "gnc_reconstruct_device_noalloc": (c_int, [ctypes.POINTER(GncConfig), c_void, c_void,
                                               c_void]),
    "gnc_filter_device": (c_int, [c_size, c_size, c_size, c_void, c_void]),
    "gnc_correct": (c_int, [c_void, c_void, c_void, c_size, c_size, c_size]),
    "gnc_get_electron_wavelength": (c_double, [c_double]),
    "gnc_get_defocus_spread": (c_double, [c_double, c_double, c_double, c_double]),
    "gnc_q_to_Q": (c_double, [c_double, c_double, c_double]),
    "gnc_Q_to_q": (c_double, [c_double, c_double, c_double]),
    "gnc_df_to_D": (c_double, [c_double, c_double, c_double]),
    "gnc_D_to_df": (c_double, [c_double, c_double, c_double]),
    "gnc_ctf_chi": (c_double, [ctypes.POINTER(GncCtf), c_double, c_double]),
    "gnc_ctf_eval": (c_int, [ctypes.POINTER(GncCtf), c_int, c_void, c_void, c_size, c_void]),
    "gnc_ctf_grid": (c_int, [ctypes.POINTER(GncCtf), c_int, c_size, c_size, c_double, c_void]),
    "gnc_q_and_theta": (c_int, [c_size, c_size, c_double, c_void, c_void]),
    "gnc_ctf_image_device": (c_int, [ctypes.POINTER(GncCtf), c_int, c_void, c_int, c_size,
                                     c_size, c_double, c_void, c_void]),
    "gnc_fbp_plan_create": (c_int, [ctypes.POINTER(GncFbpDesc), ctypes.POINTER(c_void)]),
    "gnc_fbp_plan_destroy": (c_int, [c_void]),
    "gnc_fbp_workspace_bytes": (c_size, [c_void]),
    "gnc_fbp_execute": (c_int, [c_void, c_void, c_void, c_void]),
    "gnc_fbp_execute_host": (c_int, [c_void, c_void, c_void, c_void]),
    "gnc_host_alloc": (c_int, [c_size, ctypes.POINTER(c_void)]),
    "gnc_host_free": (c_int, [c_void]),
    "gnc_fbp_correct": (c_int, [c_void, c_void, c_void, c_void]),
    "gnc_fbp_stage": (c_int, [c_void, c_void, c_void]),
    "gnc_fbp_backproject": (c_int, [c_void, c_void, c_int, c_void]),
    "gnc_fbp_backproject_staged": (c_int, [c_void, c_void, c_void, c_void, c_int, c_void]),
    "gnc_fbp_slab_map": (c_int, [c_void, c_void, c_void]),
    "gnc_fbp_sign_table": (c_int, [c_void, c_void, c_void]),
    "gnc_fbp_staged": (c_int, [c_void, ctypes.POINTER(c_void), ctypes.POINTER(c_void)]),
    "gnc_fbp_check": (c_int, [c_void, c_void]),
    "gnc_fbp_launches": (c_int, [c_void]),
    "gnc_fbp_backprojector": (c_int, [c_void]),
    "gnc_fbp_live_slabs": (c_int, [c_void, c_void, c_void]),
    "gnc_debug_wait_probe": (c_int, [ctypes.c_uint]),
    "gnc_server_create": (c_int, [c_size, c_int, ctypes.POINTER(c_void)]),
    "gnc_server_destroy": (c_int, [c_void]),
    "gnc_server_submit": (c_int, [c_void, ctypes.POINTER(GncFbpDesc), c_void, c_void,
                                  ctypes.POINTER(ctypes.c_uint64)]),
    "gnc_server_wait": (c_int, [c_void, ctypes.c_uint64, c_double,
                                ctypes.POINTER(GncRequestInfo)]),
    "gnc_server_wait_any": (c_int, [c_void, c_double, ctypes.POINTER(ctypes.c_uint64),
                                    ctypes.POINTER(GncRequestInfo)]),
    "gnc_server_now": (c_double, [c_void]),
    "gnc_server_get_stats": (c_int, [c_void, ctypes.POINTER(GncServerStats)]),
}


class GncError(RuntimeError):
    """A failed C ABI call; the message is gnc_last_error()."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (and bind) the library; raises if it cannot be loaded."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is not built; run `python -m guanaco_gb300.build`")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def check(status):
    if status != GNC_OK:
        msg = load().gnc_last_error().decode(errors="replace")
        raise GncError(status, msg)
