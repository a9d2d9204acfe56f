"""Render entry points (core/render.py of the reference) over the C ABI.

``render``, ``render_response_matrix`` and ``render_debug`` keep the
reference's signatures and results; the work is one call into the CUDA
library (include/iactrace_gb300.h). There is no CPU path: without a CUDA
device or without the built library these functions raise.
"""
from __future__ import annotations

import ctypes
import math

import torch

from .. import _native as N
from .scene import pack_scene, stages_of


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("iactrace_gb300 renders on a CUDA device; none is available")
    return torch.device("cuda", torch.cuda.current_device())


def source_code(source_type) -> int:
    """core/render.py:129-133: 'point' is a point source, anything else parallel."""
    return N.SRC_POINT if source_type == "point" else N.SRC_PARALLEL


def _inputs(sources, values, device):
    src = torch.as_tensor(sources).to(device=device, dtype=torch.float32).reshape(-1, 3).contiguous()
    val = torch.as_tensor(values).to(device=device, dtype=torch.float32).reshape(-1).contiguous()
    if src.shape[0] != val.shape[0]:
        raise ValueError(f"sources ({src.shape[0]}) and values ({val.shape[0]}) disagree in length")
    return src, val


def _workspace(ps, sdesc, S, mode, device):
    """Per-call scratch from torch's stream-ordered caching allocator."""
    return torch.empty(max(ps.workspace_bytes(sdesc, S, mode), 256), dtype=torch.uint8, device=device)


def _launch(tel, sources, values, source_type, sensor_idx, mode, opts=None):
    device = _device()
    sensor = tel.sensors[sensor_idx]
    src, val = _inputs(sources, values, device)
    S = int(src.shape[0])
    P = int(math.prod(sensor.get_accumulator_shape()))
    shape = (S, P) if mode == N.MODE_RESPONSE else tuple(sensor.get_accumulator_shape())
    if 0 not in stages_of(tel):  # core/render.py:197-199 empty telescope
        return torch.zeros(shape, device=device)
    lib = N.load()
    ps = pack_scene(tel, device)
    sdesc, keep = sensor.pack(device)
    out = torch.empty(shape, dtype=torch.float32, device=device)
    ws = _workspace(ps, sdesc, S, mode, device)
    stream = torch.cuda.current_stream(device).cuda_stream
    N.check(lib.iact_render(ctypes.byref(ps.desc), ctypes.byref(sdesc), source_code(source_type),
                            src.data_ptr(), val.data_ptr(), S, mode, out.data_ptr(), ws.data_ptr(),
                            ws.numel(), ctypes.byref(opts) if opts is not None else None, stream))
    del keep
    return out


def render(tel, sources, values, source_type="point", sensor_idx=0, opts=None):
    """core/render.py:174-220: image with the sensor's accumulator shape."""
    return _launch(tel, sources, values, source_type, sensor_idx, N.MODE_IMAGE, opts)


def render_response_matrix(tel, sources, values, source_type="point", sensor_idx=0, opts=None):
    """core/render.py:271-324: (n_sources, n_pixels) per-source rows."""
    return _launch(tel, sources, values, source_type, sensor_idx, N.MODE_RESPONSE, opts)


def render_debug(tel, sources, values, source_type="point", sensor_idx=0, extras=False):
    """core/render.py:223-268: raw hits (F*S*M, 2) and values (F*S*M,), ray
    order (facet, source, sample). With extras=True also the hard pixel id
    and the index of the last stage mirror hit per ray."""
    device = _device()
    sensor = tel.sensors[sensor_idx]
    src, val = _inputs(sources, values, device)
    S = int(src.shape[0])
    if 0 not in stages_of(tel):
        z = (torch.zeros((0, 2), device=device), torch.zeros((0,), device=device))
        return z + (torch.zeros(0, dtype=torch.int32, device=device),) * 2 if extras else z
    lib = N.load()
    ps = pack_scene(tel, device)
    sdesc, keep = sensor.pack(device)
    n = ps.F * S * ps.M
    pts = torch.empty((n, 2), dtype=torch.float32, device=device)
    vals = torch.empty((n,), dtype=torch.float32, device=device)
    pix = torch.empty((n,), dtype=torch.int32, device=device) if extras else None
    hm = torch.empty((n,), dtype=torch.int32, device=device) if extras else None
    ws = _workspace(ps, sdesc, S, N.MODE_DEBUG, device)
    stream = torch.cuda.current_stream(device).cuda_stream
    N.check(lib.iact_render_debug(ctypes.byref(ps.desc), ctypes.byref(sdesc), source_code(source_type),
                                  src.data_ptr(), val.data_ptr(), S, pts.data_ptr(), vals.data_ptr(),
                                  pix.data_ptr() if extras else None, hm.data_ptr() if extras else None,
                                  ws.data_ptr(), ws.numel(), stream))
    del keep
    return (pts, vals, pix, hm) if extras else (pts, vals)
