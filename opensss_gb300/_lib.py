"""ctypes binding of ``libsss300.so`` (the C ABI declared in ``include/sss300.h``).

There is no CPU fallback: if the library is missing or cannot be loaded every
entry point raises ``EngineUnavailable``.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsss300.so")

SSS_OK = 0
ABI_VERSION = 7  # SSS300_ABI_VERSION of include/sss300.h
ERROR_NAMES = {
    1: "SSS_ERR_INVALID", 2: "SSS_ERR_CUDA", 3: "SSS_ERR_OVERRUN", 4: "SSS_ERR_TOF_RANGE",
    5: "SSS_ERR_ENERGY", 6: "SSS_ERR_VOXEL", 7: "SSS_ERR_WORKSPACE", 8: "SSS_ERR_CAPACITY",
    9: "SSS_ERR_EVENT", 10: "SSS_ERR_NONFINITE", 11: "SSS_ERR_TABLE",
}

# every symbol the header declares, with (restype, argtypes)
_P = C.c_void_p
_I32, _I64, _D = C.c_int32, C.c_int64, C.c_double


class EngineUnavailable(RuntimeError):
    """The compiled sm_103a engine is not available."""


class SSSError(RuntimeError):
    def __init__(self, code: int, message: str):
        self.code = code
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")


class TofProblem(C.Structure):
    """Mirror of ``struct sss_tof_problem``."""
    _fields_ = [
        ("nx", _I32), ("ny", _I32), ("nz", _I32),
        ("activity", _P), ("attenuation", _P),
        ("image_size", _D * 6),
        ("nr", _I32), ("nd", _I32),
        ("geometry", _P), ("normals", _P),
        ("detector_size", _D * 2),
        ("nru", _I32), ("ndu", _I32),
        ("rings", _P), ("detectors", _P),
        ("sample_step", _I32 * 3),
        ("nbins", _I32),
        ("tof_bin_width", _D), ("tof_resolution", _D),
        ("tof_log2w", _P), ("efficiency", _P), ("atten_ratio", _P),
        ("flags", _I32),
        ("pair_warps", _I32), ("leg_threads", _I32),
    ]


SSS_FLAG_KAHAN = 1
SSS_FLAG_UNIT_TOF = 2


class ListmodeLayout(C.Structure):
    """Mirror of ``struct sss_listmode_layout``."""
    _fields_ = [("record_bytes", _I32), ("id_offset", _I32), ("tof_offset", _I32),
                ("scatter_offset", _I32)]


class SinoMap(C.Structure):
    """Mirror of ``struct sss_sino_map``."""
    _fields_ = [("lor", _P), ("nd_lor", _I32), ("mash", _I32), ("shift", _I32), ("slices", _P),
                ("nr_table", _I32), ("nrad", _I32), ("nang", _I32), ("nslices", _I32),
                ("tof_bins", _I32), ("tof_range", _D)]


SIGNATURES = {
    "sss_last_error": (C.c_char_p, []),
    "sss_abi_version": (C.c_int, []),
    "sss_status_code": (C.c_int, [_I32]),
    "sss_raytrace": (C.c_int, [_P, _P, _P, _I64, _I32, _I32, _P, _P, _P, _P, _P, _P, _P]),
    "sss_scatter_points": (C.c_int, [C.POINTER(TofProblem), _P, _I64, C.POINTER(_I64), _P, _P]),
    "sss_scatter_points_noalloc": (C.c_int, [C.POINTER(TofProblem), _P, _I64, C.POINTER(_I64), _P,
                                             _P]),
    "sss_tof_workspace_size": (C.c_size_t, [C.POINTER(TofProblem), _I64]),
    "sss_tof_run": (C.c_int, [C.POINTER(TofProblem), _P, _I64, _P, _I64, _I64, _P, C.c_size_t,
                              _P, _P, _P]),
    "sss_tof_densify": (C.c_int, [_P, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _P]),
    "sss_tof_densify_full": (C.c_int, [_P, _I32, _I32, _I32, _I32, _P, _P, _P, _P]),
    "sss_tof_densify_cells": (C.c_int, [_P, _I32, _I32, _I32, _I32, _P, _P, _P, _P]),
    "sss_batch_plan": (C.c_int, [C.POINTER(TofProblem), _I32, _P, _P, C.c_size_t, _P,
                                 C.POINTER(_P), _P]),
    "sss_batch_run": (C.c_int, [_P, _P]),
    "sss_batch_plan_points": (C.c_int, [C.POINTER(TofProblem), _I32, _P, _P, _P, _P, C.c_size_t, _P,
                                        C.POINTER(_P), _P]),
    "sss_batch_run_waves": (C.c_int, [_P, _I32, _I32, _P]),
    "sss_batch_info": (C.c_int, [_P, _P]),
    "sss_batch_free": (None, [_P]),
    "sss_upsample": (C.c_int, [_P, _I64, _I32, _P, _I64, _P, _I32, _P, _I32, _P, _P]),
    "sss_tail_mask": (C.c_int, [_P, _P, _P, _I32, _I32, _I32, _P, _P, _P, _I32, _D, _P, _P, _P]),
    "sss_tail_mask_pairs": (C.c_int, [_P, _P, _P, _I32, _I32, _I32, _P, _P, _P, _I32, _I32, _I32, _D, _P,
                                      _P, _P]),
    "sss_backproject_fit_pairs": (C.c_int, [_P, _P, _I32, _I32, _P, _P, _P, _I32, _I32, _I32, _I32, _P, _P,
                                            _P, _P, _P, _P, _P, _I32, _P, _P, _P, _P, _P]),
    "sss_backproject_fit": (C.c_int, [_P, _P, _I32, _I32, _P, _P, _P, _I32, _P, _P, _P, _P, _P, _P,
                                      _P, _I32, _P, _P, _P, _P, _P]),
    "sss_backproject_fit_bins": (C.c_int, [_P, _P, _I32, _I32, _P, _P, _P, _P, _I32, _I32, _I32, _I32, _I32,
                                           _P, _I64, _P, _P, _P, _P, _I64, _P, _P, _I32, _P, _P, _P, _P, _P]),
    "sss_histogram_prompts": (C.c_int, [_P, _I64, C.POINTER(ListmodeLayout), C.POINTER(SinoMap), _P, _P,
                                        _P, _P]),
    "sss_histogram_finish": (C.c_int, [_P, _I64, C.POINTER(ListmodeLayout), C.POINTER(SinoMap), _P, _P,
                                       _D, _P, _P, _P, _P]),
    "sss_inject_workspace_size": (C.c_size_t, [_I64]),
    "sss_inject_scatters": (C.c_int, [_P, _I64, C.POINTER(ListmodeLayout), C.POINTER(SinoMap), _P, _P,
                                      _P, _P, _P, C.c_size_t, _P, _P]),
    "sss_crop_downscale_workspace_size": (C.c_size_t, [_P]),
    "sss_crop_downscale": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.c_int, C.c_float, _P, _P, C.c_size_t, _P]),
    "sss_pair_warps_max": (C.c_int, [_I32, _I32]),
    "sss_set_timing": (None, [C.c_int]),
    "sss_get_timing": (C.c_int, [_P]),
}

_lib = None
_lock = threading.Lock()


def lib():
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise EngineUnavailable(
                    f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
            try:
                h = C.CDLL(LIB_PATH)
            except OSError as e:  # wrong architecture, missing libcudart, ...
                raise EngineUnavailable(f"cannot load {LIB_PATH}: {e}") from e
            for name, (res, args) in SIGNATURES.items():
                try:
                    f = getattr(h, name)
                except AttributeError as e:
                    raise EngineUnavailable(f"{LIB_PATH} is stale (no {name}); rebuild it") from e
                f.restype = res
                f.argtypes = args
            if h.sss_abi_version() != ABI_VERSION:
                raise EngineUnavailable(f"{LIB_PATH} has ABI {h.sss_abi_version()}, expected {ABI_VERSION}; "
                                        "rebuild it")
            _lib = h
    return _lib


def require_cuda(**tensors) -> None:
    """Raise ValueError unless every given tensor (None skipped) lives on a
    CUDA device: the kernels take raw device pointers, and a host pointer would
    reach the GPU unchecked."""
    for name, t in tensors.items():
        if t is not None and not (hasattr(t, "is_cuda") and t.is_cuda):
            raise ValueError(f"{name} must be a CUDA tensor")


def last_error() -> str:
    return lib().sss_last_error().decode(errors="replace")


def check(rc: int):
    if rc != SSS_OK:
        raise SSSError(rc, last_error())


def check_status(status_word: int):
    """Raise for a non-zero device status word (after synchronisation)."""
    if status_word:
        rc = lib().sss_status_code(int(status_word))
        check(rc)
