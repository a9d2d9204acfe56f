"""ORACLE — test infrastructure only. ctypes front end of the C++ restatement
(iact_oracle.hpp): FP64 oracle and FP32 restatement of the reference render
path, fed the same packed tables as the CUDA library (host copies).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use this module, as the oracle of the parity tests and as the timed CPU
restatement.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("iact_oracle.cpp", "iact_oracle.hpp")]
    srcs.append(os.path.join(os.path.dirname(HERE), "include", "iactrace_gb300.h"))
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-o", LIB + ".tmp",
           os.path.join(HERE, "iact_oracle.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        vp, i, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32
        for name in ("oracle_render_f64", "oracle_render_f32"):
            getattr(lib, name).argtypes = [vp, vp, i, vp, vp, i, i, vp, i, u]
            getattr(lib, name).restype = i
        for name in ("oracle_render_debug_f64", "oracle_render_debug_f32"):
            getattr(lib, name).argtypes = [vp, vp, i, vp, vp, i, vp, vp, vp, vp, vp, u]
            getattr(lib, name).restype = i
        lib.oracle_transform_f64.argtypes = [vp, vp, vp, vp]
        lib.oracle_sample_facets.argtypes = [vp, vp, vp, vp, vp]
        lib.oracle_sample_facets.restype = i
        lib.oracle_max_threads.restype = i
        _lib = lib
    return _lib


def _host(tel, sensor_idx):
    from iactrace_gb300.core.scene import pack_scene
    ps = pack_scene(tel, "cpu")
    sdesc, keep = tel.sensors[sensor_idx].pack("cpu")
    return ps, sdesc, keep


def _src(sources, values, source_type="point"):
    width = 4 if source_type == "extended" else 3
    s = np.ascontiguousarray(torch.as_tensor(sources).detach().cpu().float().numpy().reshape(-1, width))
    v = np.ascontiguousarray(torch.as_tensor(values).detach().cpu().float().numpy().reshape(-1))
    return s, v


def source_code(source_type) -> int:
    return {"point": 0, "extended": 2}.get(source_type, 1)


def render(tel, sources, values, source_type="point", sensor_idx=0, mode="image", dtype="f64", threads=1, seed=0):
    """Image (accumulator shape) or response matrix (S, P) from the oracle."""
    lib = load()
    ps, sd, keep = _host(tel, sensor_idx)
    s, v = _src(sources, values, source_type)
    S = s.shape[0]
    P = int(math.prod(tel.sensors[sensor_idx].get_accumulator_shape()))
    m = 1 if mode == "response" else 0
    npd = np.float64 if dtype == "f64" else np.float32
    out = np.zeros((S, P) if m else (P,), npd)
    fn = lib.oracle_render_f64 if dtype == "f64" else lib.oracle_render_f32
    if ps.F and ps.M:
        rc = fn(ctypes.addressof(ps.desc), ctypes.addressof(sd), source_code(source_type), s.ctypes.data,
                v.ctypes.data, S, m, out.ctypes.data, threads, seed)
        if rc:
            raise RuntimeError(f"oracle render failed: {rc}")
    del keep
    return out if m else out.reshape(tel.sensors[sensor_idx].get_accumulator_shape())


def render_debug(tel, sources, values, source_type="point", sensor_idx=0, dtype="f64", seed=0):
    """Per-ray (x, y), value, hard pixel id, last stage-mirror hit, pixel-edge margin."""
    lib = load()
    ps, sd, keep = _host(tel, sensor_idx)
    s, v = _src(sources, values, source_type)
    S = s.shape[0]
    n = ps.F * S * ps.M
    npd = np.float64 if dtype == "f64" else np.float32
    pts = np.zeros((n, 2), npd)
    vals = np.zeros(n, npd)
    pix = np.zeros(n, np.int32)
    hm = np.zeros(n, np.int32)
    mg = np.zeros(n, npd)
    fn = lib.oracle_render_debug_f64 if dtype == "f64" else lib.oracle_render_debug_f32
    if n:
        rc = fn(ctypes.addressof(ps.desc), ctypes.addressof(sd), source_code(source_type), s.ctypes.data,
                v.ctypes.data, S, pts.ctypes.data, vals.ctypes.data, pix.ctypes.data, hm.ctypes.data, mg.ctypes.data,
                seed)
        if rc:
            raise RuntimeError(f"oracle debug failed: {rc}")
    del keep
    return {"pts": pts, "vals": vals, "pix": pix, "hit_mirror": hm, "margin": mg}


def max_threads() -> int:
    return int(load().oracle_max_threads())


def sample_facets(sampler_desc, F: int, M: int):
    """Replay of iact_sample_facets on host arrays (the descriptor's array
    pointers must be host pointers): points, normals, delta [F, M, 3] and
    weights [F, M], float64."""
    lib = load()
    pts, nrm, dlt = (np.zeros((F, M, 3)) for _ in range(3))
    wts = np.zeros((F, M))
    rc = lib.oracle_sample_facets(ctypes.addressof(sampler_desc), pts.ctypes.data, nrm.ctypes.data,
                                  dlt.ctypes.data, wts.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_sample_facets failed ({rc})")
    return pts, nrm, dlt, wts
