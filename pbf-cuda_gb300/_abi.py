"""ctypes binding of libpbf.so (include/pbf.h).

The library is the product: there is no fallback.  If libpbf.so is missing it
is built with nvcc (build.py); if that fails, import of the binding raises.
"""
from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

from . import build as _build

PBF_OK = 0
PBF_ERR_INVALID_ARG = 1
PBF_ERR_CAPACITY = 2
PBF_ERR_CUDA = 3
PBF_ERR_TIMEOUT = 4
PBF_ERR_NOT_READY = 5

# Largest max_particles of a solver / total of a batch (32-bit table indices).
PBF_MAX_PARTICLES = 1 << 27

# Every symbol include/pbf.h declares, in declaration order.
EXPORTED = (
    "pbf_params_default",
    "pbf_status_string",
    "pbf_last_error",
    "pbf_abi_version",
    "pbf_create",
    "pbf_destroy",
    "pbf_set_params",
    "pbf_get_params",
    "pbf_set_limits",
    "pbf_get_limits",
    "pbf_step",
    "pbf_get_density",
    "pbf_build_grid",
    "pbf_profile_enable",
    "pbf_profile_read",
    "pbf_use_graphs",
    "pbf_tape_enable",
    "pbf_backward",
    "pbf_density_grid",
    "pbf_density_grid_backward",
    "pbf_batch_create",
    "pbf_batch_destroy",
    "pbf_batch_set_limits",
    "pbf_batch_step",
    "pbf_batch_get_density",
    "pbf_batch_use_graphs",
    "pbf_autotune",
    "pbf_batch_autotune",
    "pbf_set_tuning",
    "pbf_get_tuning",
    "pbf_batch_set_tuning",
    "pbf_batch_get_tuning",
    "pbf_check_device",
    "pbf_batch_check_device",
    "pbf_step_noalloc",
)

# Every symbol include/pbf_ssf.h declares, in declaration order.
EXPORTED_SSF = (
    "pbf_ssf_params_default",
    "pbf_ssf_look_at",
    "pbf_ssf_create",
    "pbf_ssf_destroy",
    "pbf_ssf_set_params",
    "pbf_ssf_get_params",
    "pbf_ssf_set_sky",
    "pbf_ssf_render",
    "pbf_ssf_images",
    "pbf_ssf_profile_enable",
    "pbf_ssf_profile_read",
)


class PbfParams(ctypes.Structure):
    """Mirror of ``pbf_params``; field names follow the reference's GUIParams
    solver fields (fluids/GUIParams.h:6-17)."""

    _fields_ = [
        ("niter", ctypes.c_int),
        ("pho0", ctypes.c_float),
        ("g", ctypes.c_float),
        ("h", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("lambda_eps", ctypes.c_float),
        ("delta_q", ctypes.c_float),
        ("k_corr", ctypes.c_float),
        ("n_corr", ctypes.c_float),
        ("k_boundaryDensity", ctypes.c_float),
        ("c_XSPH", ctypes.c_float),
        ("up", ctypes.c_float * 3),
        ("lim_eps", ctypes.c_float),
        ("kernel_eps", ctypes.c_float),
        ("max_dp", ctypes.c_float),
        ("vorticity_eps", ctypes.c_float),
    ]

    def copy(self) -> "PbfParams":
        out = PbfParams()
        ctypes.pointer(out)[0] = self
        return out

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = [float(x) for x in v] if name == "up" else v
        return d

    def __repr__(self) -> str:
        return "PbfParams(" + ", ".join(f"{k}={v!r}" for k, v in self.as_dict().items()) + ")"


class PbfStepProfile(ctypes.Structure):
    """Mirror of ``pbf_step_profile``."""

    _fields_ = [
        ("grid_ms", ctypes.c_float),
        ("reorder_ms", ctypes.c_float),
        ("lambda_ms", ctypes.c_float),
        ("delta_p_ms", ctypes.c_float),
        ("xsph_ms", ctypes.c_float),
        ("total_ms", ctypes.c_float),
        ("iterations", ctypes.c_int),
        ("launches", ctypes.c_int),
        ("grid_launches", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class PbfTuning(ctypes.Structure):
    """Mirror of ``pbf_tuning`` (include/pbf.h)."""

    _fields_ = [("dense_window", ctypes.c_int), ("dense_all", ctypes.c_int),
                ("ms_per_step", ctypes.c_float), ("ms_default", ctypes.c_float), ("order", ctypes.c_int),
                ("bwd_lanes", ctypes.c_int), ("stage_sparse", ctypes.c_int), ("stage_dense", ctypes.c_int),
                ("queue_sparse", ctypes.c_int), ("queue_dense", ctypes.c_int), ("dense_split", ctypes.c_int),
                ("dense_interleave", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PbfSsfParams(ctypes.Structure):
    """Mirror of ``pbf_ssf_params`` (include/pbf_ssf.h); renderer fields follow
    the reference's GUIParams renderer fields (fluids/GUIParams.h:19-38)."""

    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("view", ctypes.c_float * 16), ("proj", ctypes.c_float * 16),
        ("p_n", ctypes.c_float), ("p_f", ctypes.c_float), ("p_t", ctypes.c_float), ("p_r", ctypes.c_float),
        ("radius", ctypes.c_float),
        ("smooth_niter", ctypes.c_int), ("kernel_r", ctypes.c_int),
        ("sigma_r", ctypes.c_float), ("sigma_z", ctypes.c_float),
        ("keep_edge", ctypes.c_int), ("blur_option", ctypes.c_int), ("shading_option", ctypes.c_int),
        ("r0", ctypes.c_float), ("sky", ctypes.c_float * 3),
    ]

    def copy(self) -> "PbfSsfParams":
        out = PbfSsfParams()
        ctypes.pointer(out)[0] = self
        return out


class PbfSsfProfile(ctypes.Structure):
    """Mirror of ``pbf_ssf_profile``."""

    _fields_ = [
        ("splat_ms", ctypes.c_float), ("smooth_ms", ctypes.c_float), ("normal_ms", ctypes.c_float),
        ("shade_ms", ctypes.c_float), ("total_ms", ctypes.c_float), ("launches", ctypes.c_int),
        ("fragments", ctypes.c_longlong),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class PbfError(RuntimeError):
    """A pbf_* call returned a status other than PBF_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} [status {status}]")
        self.status = status


_lock = threading.Lock()
_lib = None


def _declare(L) -> None:
    P = ctypes.POINTER
    f3 = P(ctypes.c_float)
    vp = ctypes.c_void_p
    u32p = P(ctypes.c_uint32)
    sig = {
        "pbf_params_default": (None, [P(PbfParams)]),
        "pbf_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "pbf_last_error": (ctypes.c_char_p, []),
        "pbf_abi_version": (ctypes.c_int, []),
        "pbf_create": (ctypes.c_int, [P(PbfParams), f3, f3, ctypes.c_int, P(vp)]),
        "pbf_destroy": (ctypes.c_int, [vp]),
        "pbf_set_params": (ctypes.c_int, [vp, P(PbfParams)]),
        "pbf_get_params": (ctypes.c_int, [vp, P(PbfParams)]),
        "pbf_set_limits": (ctypes.c_int, [vp, f3, f3]),
        "pbf_get_limits": (ctypes.c_int, [vp, f3, f3]),
        "pbf_step": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, ctypes.c_int, vp]),
        "pbf_get_density": (ctypes.c_int, [vp, vp, ctypes.c_int, vp]),
        "pbf_build_grid": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, vp, vp, vp, P(ctypes.c_int), vp]),
        "pbf_profile_enable": (ctypes.c_int, [vp, ctypes.c_int]),
        "pbf_profile_read": (ctypes.c_int, [vp, P(PbfStepProfile)]),
        "pbf_use_graphs": (ctypes.c_int, [vp, ctypes.c_int]),
        "pbf_tape_enable": (ctypes.c_int, [vp, ctypes.c_int]),
        "pbf_backward": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
        "pbf_density_grid": (ctypes.c_int, [vp, ctypes.c_int, f3, f3, P(ctypes.c_int), ctypes.c_float, vp, vp]),
        "pbf_density_grid_backward": (ctypes.c_int, [vp, ctypes.c_int, f3, f3, P(ctypes.c_int), ctypes.c_float, vp,
                                                     vp, vp]),
        "pbf_batch_create": (ctypes.c_int, [P(PbfParams), ctypes.c_int, f3, f3, P(ctypes.c_int), P(vp)]),
        "pbf_batch_destroy": (ctypes.c_int, [vp]),
        "pbf_batch_set_limits": (ctypes.c_int, [vp, ctypes.c_int, f3, f3]),
        "pbf_batch_step": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
        "pbf_batch_get_density": (ctypes.c_int, [vp, vp, vp]),
        "pbf_batch_use_graphs": (ctypes.c_int, [vp, ctypes.c_int]),
        "pbf_autotune": (ctypes.c_int, [vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp]),
        "pbf_batch_autotune": (ctypes.c_int, [vp, vp, vp, vp, ctypes.c_int, vp, vp]),
        "pbf_set_tuning": (ctypes.c_int, [vp, P(PbfTuning)]),
        "pbf_get_tuning": (ctypes.c_int, [vp, P(PbfTuning)]),
        "pbf_batch_set_tuning": (ctypes.c_int, [vp, P(PbfTuning)]),
        "pbf_batch_get_tuning": (ctypes.c_int, [vp, P(PbfTuning)]),
        "pbf_check_device": (ctypes.c_int, [vp, vp]),
        "pbf_batch_check_device": (ctypes.c_int, [vp, vp]),
        "pbf_step_noalloc": (ctypes.c_int, [P(PbfParams), f3, f3, vp, vp, vp, vp, vp, ctypes.c_int, vp]),
        "pbf_ssf_params_default": (None, [P(PbfSsfParams)]),
        "pbf_ssf_look_at": (ctypes.c_int, [P(PbfSsfParams), f3, f3, ctypes.c_float]),
        "pbf_ssf_create": (ctypes.c_int, [P(PbfSsfParams), P(vp)]),
        "pbf_ssf_destroy": (None, [vp]),
        "pbf_ssf_set_params": (ctypes.c_int, [vp, P(PbfSsfParams)]),
        "pbf_ssf_get_params": (ctypes.c_int, [vp, P(PbfSsfParams)]),
        "pbf_ssf_set_sky": (ctypes.c_int, [vp, f3, ctypes.c_int]),
        "pbf_ssf_render": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, vp]),
        "pbf_ssf_images": (ctypes.c_int, [vp, vp, vp, vp, vp]),
        "pbf_ssf_profile_enable": (ctypes.c_int, [vp, ctypes.c_int]),
        "pbf_ssf_profile_read": (ctypes.c_int, [vp, P(PbfSsfProfile)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib_path():
    return Path(os.environ["PBF_LIB"]) if os.environ.get("PBF_LIB") else _build.LIB


def lib():
    """Load (building first if needed) libpbf.so; PBF_LIB names another build of it."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path() if os.environ.get("PBF_LIB") else _build.build()
            L = ctypes.CDLL(str(path))
            _declare(L)
            _lib = L
    return _lib


def check(status: int, what: str = "pbf call") -> None:
    if status != PBF_OK:
        L = lib()
        msg = L.pbf_last_error().decode(errors="replace")
        name = L.pbf_status_string(status).decode()
        raise PbfError(status, f"{what}: {name}: {msg}")


def default_params() -> PbfParams:
    """The reference's defaults (fluids/FluidSystem.cpp:15-25, fluids/helper.h:4-9)."""
    p = PbfParams()
    lib().pbf_params_default(ctypes.byref(p))
    return p
