"""ctypes binding of the C ABI (include/iactrace_gb300.h).

The structs below mirror the header field by field; ``check_layout`` compares
their sizes with what the compiled library reports. Every entry point returns
an IACT status; a non-zero status raises :class:`IactError` with the
library's thread-local message. There is no fallback: without the compiled
library the render path raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

IACT_OK = 0
IACT_E_INVALID = -1
IACT_E_UNSUPPORTED = -2
IACT_E_CUDA = -3
IACT_E_WORKSPACE = -4
IACT_E_DEVICE = -5

IACT_MAX_ASPH = 8
IACT_MAX_POLY = 8
IACT_MAX_STAGE_MIRRORS = 64
IACT_MAX_OBSTRUCTIONS = 2048

SRC_POINT = 0
SRC_PARALLEL = 1
SRC_EXTENDED = 2
MODE_IMAGE = 0
MODE_RESPONSE = 1
MODE_DEBUG = 2
MODE_BACKWARD = 3
SENSOR_SQUARE = 0
SENSOR_HEX = 1
SENSOR_SOFT_SQUARE = 2
SENSOR_SOFT_HEX = 3
FLAG_NO_CULL = 1
FLAG_BATCH_BACKWARD = 2
APERTURE_DISK = 0
APERTURE_POLYGON = 1

_f = ctypes.c_float
_i = ctypes.c_int32
_pf = ctypes.POINTER(ctypes.c_float)
_pi = ctypes.POINTER(ctypes.c_int32)


class IactMirror(ctypes.Structure):
    _fields_ = [
        ("stage", _i), ("aperture", _i), ("n_asph", _i), ("n_vert", _i),
        ("pos", _f * 3), ("rot", _f * 3), ("offset", _f * 2),
        ("curvature", _f), ("conic", _f),
        ("asph", _f * IACT_MAX_ASPH),
        ("radius", _f),
        ("vert", (_f * 2) * IACT_MAX_POLY),
        ("pad_", _f * 5),
    ]


class IactScene(ctypes.Structure):
    _fields_ = [
        ("n_facets", _i), ("n_samples", _i),
        ("facet_pos", ctypes.c_void_p), ("facet_rot", ctypes.c_void_p), ("facet_scale", ctypes.c_void_p),
        ("points", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("delta", ctypes.c_void_p),
        ("weights", ctypes.c_void_p),
        ("n_mirrors", _i), ("n_stages", _i), ("mirrors", ctypes.c_void_p),
        ("n_cyl", _i), ("n_box", _i), ("n_sph", _i), ("n_obox", _i), ("n_tri", _i),
        ("cyl", ctypes.c_void_p), ("box", ctypes.c_void_p), ("sph", ctypes.c_void_p),
        ("obox", ctypes.c_void_p), ("tri", ctypes.c_void_p),
    ]


class IactSensor(ctypes.Structure):
    _fields_ = [
        ("type", _i), ("n_pixels", _i), ("width", _i), ("height", _i),
        ("pos", _f * 3), ("rot", _f * 3),
        ("x0", _f), ("y0", _f), ("dx", _f), ("dy", _f), ("edge_width", _f),
        ("hex_size", _f), ("inradius", _f), ("grid_cos", _f), ("grid_sin", _f),
        ("off_x", _f), ("off_y", _f), ("hex_sx", _f), ("hex_sy", _f),
        ("edge_threshold", _f),
        ("q_min", _i), ("r_min", _i), ("table_q", _i), ("table_r", _i),
        ("table", ctypes.c_void_p),
        ("sigma", _f), ("kernel_size", _i),
    ]


class IactOpts(ctypes.Structure):
    _fields_ = [("block_threads", _i), ("sources_per_cta", _i), ("facets_per_tile", _i), ("hist_mode", _i),
                ("tasks_per_warp", _i), ("flags", _i), ("seed", ctypes.c_uint32), ("kernel_events", ctypes.c_void_p * 2)]


class IactJob(ctypes.Structure):
    _fields_ = [("scene", ctypes.POINTER(IactScene)), ("sensor", ctypes.POINTER(IactSensor)),
                ("sources", ctypes.c_void_p), ("values", ctypes.c_void_p), ("n_sources", _i),
                ("seed", ctypes.c_uint32), ("out", ctypes.c_void_p), ("grad_out", ctypes.c_void_p),
                ("g_facet_rot", ctypes.c_void_p), ("g_facet_pos", ctypes.c_void_p), ("g_facet_scale", ctypes.c_void_p),
                ("g_sources", ctypes.c_void_p), ("g_values", ctypes.c_void_p), ("g_mirror_rot", ctypes.c_void_p),
                ("g_mirror_pos", ctypes.c_void_p), ("g_mirror_surface", ctypes.c_void_p)]


class IactSampler(ctypes.Structure):
    _fields_ = [("n_facets", _i), ("n_samples", _i), ("aperture", _i), ("n_vert", _i),
                ("curvature", _f), ("conic", _f), ("n_asph", _i), ("asph", _f * IACT_MAX_ASPH),
                ("offsets", ctypes.c_void_p), ("radii", ctypes.c_void_p), ("vertices", ctypes.c_void_p),
                ("seed", ctypes.c_uint32), ("surface", ctypes.c_void_p)]


class IactError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"iactrace_gb300 error {code}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None

_SIGS = {
    "iact_abi_version": ([], ctypes.c_int),
    "iact_last_error": ([], ctypes.c_char_p),
    "iact_abi_layout": ([ctypes.POINTER(ctypes.c_size_t), ctypes.c_int], ctypes.c_int),
    "iact_workspace_size": ([ctypes.POINTER(IactScene), ctypes.POINTER(IactSensor), _i, _i,
                             ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "iact_render": ([ctypes.POINTER(IactScene), ctypes.POINTER(IactSensor), _i, ctypes.c_void_p, ctypes.c_void_p,
                     _i, _i, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(IactOpts),
                     ctypes.c_void_p], ctypes.c_int),
    "iact_probe_fma": ([ctypes.c_void_p, _i, _i, ctypes.c_void_p], ctypes.c_int),
    "iact_kernel_launches": ([], ctypes.c_int64),
    "iact_render_backward": ([ctypes.POINTER(IactScene), ctypes.POINTER(IactSensor), _i, ctypes.c_void_p,
                              ctypes.c_void_p, _i, _i, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.POINTER(IactOpts), ctypes.c_void_p], ctypes.c_int),
    "iact_render_debug": ([ctypes.POINTER(IactScene), ctypes.POINTER(IactSensor), _i, ctypes.c_void_p,
                           ctypes.c_void_p, _i, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "iact_batch_create": ([ctypes.POINTER(IactJob), _i, _i, _i, ctypes.POINTER(IactOpts),
                           ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "iact_batch_workspace_size": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "iact_batch_prepare": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p], ctypes.c_int),
    "iact_batch_render": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "iact_batch_backward": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "iact_batch_info": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), _i], ctypes.c_int),
    "iact_batch_destroy": ([ctypes.c_void_p], None),
    "iact_sample_facets": ([ctypes.POINTER(IactSampler), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "iact_sample_facets_backward": ([ctypes.POINTER(IactSampler), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
}

# symbols declared by include/iactrace_gb300.h that bindings resolve
EXPORTED = list(_SIGS.keys())


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the compiled library (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise ImportError(
                    f"iactrace_gb300 native library not built ({path}); run "
                    "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        check_layout(lib)
        return lib


def check_layout(lib) -> None:
    out = (ctypes.c_size_t * 6)()
    rc = lib.iact_abi_layout(out, 6)
    if rc != IACT_OK:
        raise IactError(rc, "iact_abi_layout failed")
    mine = [ctypes.sizeof(IactScene), ctypes.sizeof(IactSensor), ctypes.sizeof(IactMirror), ctypes.sizeof(IactOpts),
            ctypes.sizeof(IactJob), ctypes.sizeof(IactSampler)]
    if list(out) != mine:
        raise ImportError(f"ABI struct layout mismatch: library {list(out)} vs binding {mine}")


def check(rc: int) -> None:
    if rc != IACT_OK:
        msg = _lib.iact_last_error().decode() if _lib is not None else "unknown"
        raise IactError(rc, msg)
