"""iact_render_noalloc: the render for callers that cannot allocate device
memory -- their device memory belongs to another framework's pool, or they
run in a real-time acquisition loop that must not allocate while observing.
Its scratch is a fixed array inside the library, so it must give what
iact_render gives with a caller workspace, call after call, and refuse work
that does not fit.

Kept in a file of its own that pytest collects last (tests/test_zz_*), so a
failure here never stops a run before the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from iactrace_gb300 import _native as N
from iactrace_gb300 import workloads as W
from iactrace_gb300.core.render import source_code
from iactrace_gb300.core.scene import pack_scene

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5  # the image tolerance of the forward parity tests


def _scratch_bytes():
    """IACT_NOALLOC_SCRATCH_BYTES as the C header defines it."""
    import os
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "iactrace_gb300.h")
    m = re.search(r"#define IACT_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", open(hdr).read())
    return int(m.group(1)) << int(m.group(2))


def _bind(lib):
    fn = lib.iact_render_noalloc
    fn.argtypes = [ctypes.POINTER(N.IactScene), ctypes.POINTER(N.IactSensor), ctypes.c_int32, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(N.IactOpts),
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _with_workspace(lib, ps, sd, st, src, val, mode, shape, stream):
    ws = torch.empty(ps.workspace_bytes(sd, src.shape[0], mode), dtype=torch.uint8, device=src.device)
    out = torch.empty(shape, device=src.device)
    N.check(lib.iact_render(ctypes.byref(ps.desc), ctypes.byref(sd), source_code(st), src.data_ptr(),
                            val.data_ptr(), src.shape[0], mode, out.data_ptr(), ws.data_ptr(), ws.numel(), None,
                            stream))
    return out


@pytest.mark.parametrize("mode", [N.MODE_IMAGE, N.MODE_RESPONSE])
def test_noalloc_matches_workspace_render_twice(cuda, mode):
    lib = N.load()
    fn = _bind(lib)
    tel, src, val, st = W.plain_forward(n_samples=128, n_sources=8)
    ps = pack_scene(tel, cuda)
    sd, keep = tel.sensors[0].pack(cuda)
    src, val = src.to(cuda).contiguous(), val.to(cuda).contiguous()
    P = tel.sensors[0].n_pixels
    shape = (src.shape[0], P) if mode == N.MODE_RESPONSE else (P,)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    ref = _with_workspace(lib, ps, sd, st, src, val, mode, shape, stream).double().cpu().numpy()
    assert np.abs(ref).sum() > 0
    for call in range(2):  # the second call starts from the first call's leftovers
        out = torch.full(shape, float("nan"), device=cuda)
        rc = fn(ctypes.byref(ps.desc), ctypes.byref(sd), source_code(st), src.data_ptr(), val.data_ptr(),
                src.shape[0], mode, out.data_ptr(), None, stream)
        assert rc == N.IACT_OK, lib.iact_last_error()
        got = out.double().cpu().numpy()
        assert np.isfinite(got).all(), f"call {call}: entries left unwritten"
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= IMG_TOL, f"call {call}: relative L2 {err:.3g} against iact_render"
    del keep


def test_noalloc_rejects_work_beyond_its_scratch(cuda):
    lib = N.load()
    fn = _bind(lib)
    tel, src, val, st = W.response_matrix(n_samples=8, n_side=64)  # 4096 x 2048 FP64 accumulator
    ps = pack_scene(tel, cuda)
    sd, keep = tel.sensors[0].pack(cuda)
    src, val = src.to(cuda).contiguous(), val.to(cuda).contiguous()
    out = torch.zeros((src.shape[0], tel.sensors[0].n_pixels), device=cuda)
    rc = fn(ctypes.byref(ps.desc), ctypes.byref(sd), source_code(st), src.data_ptr(), val.data_ptr(),
            src.shape[0], N.MODE_RESPONSE, out.data_ptr(), None, torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == N.IACT_E_UNSUPPORTED
    assert b"scratch" in lib.iact_last_error()
    assert float(out.abs().sum()) == 0.0  # nothing was queued
    del keep


LIMIT = _scratch_bytes()


def _largest_fitting_sources(lib, ps, sd, mode):
    """The largest source count whose scratch fits the fixed array."""
    def need(S):
        size = ctypes.c_size_t(0)
        N.check(lib.iact_workspace_size(ctypes.byref(ps.desc), ctypes.byref(sd), int(S), mode, ctypes.byref(size)))
        return int(size.value)
    lo, hi = 1, 1
    while need(hi) <= LIMIT:
        lo, hi = hi, hi * 2
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if need(mid) <= LIMIT else (lo, mid)
    return lo, need(lo), need(lo + 1)


def test_noalloc_at_the_limit_with_options(cuda):
    """A response render whose scratch just fits the array gives what
    iact_render gives (also with non-default launch options: 128 threads per
    CTA), and one source more is refused before anything is queued."""
    lib = N.load()
    fn = _bind(lib)
    tel, _, _, st = W.plain_forward(n_samples=16, n_sources=1)
    ps = pack_scene(tel, cuda)
    sd, keep = tel.sensors[0].pack(cuda)
    S, need, need_more = _largest_fitting_sources(lib, ps, sd, N.MODE_RESPONSE)
    assert need <= LIMIT < need_more
    assert need > LIMIT - 16 * 1024  # within one output row or so of the limit
    src = W.point_sources_disk(S + 1, 2.5, 3).to(cuda).contiguous()
    val = (torch.rand(S + 1, generator=torch.Generator().manual_seed(4)) + 0.5).to(cuda).contiguous()
    P = tel.sensors[0].n_pixels
    stream = torch.cuda.current_stream(cuda).cuda_stream
    ref = _with_workspace(lib, ps, sd, st, src[:S], val[:S], N.MODE_RESPONSE, (S, P), stream).double().cpu().numpy()
    opts = N.IactOpts()
    opts.block_threads = 128
    for o in (None, opts):
        out = torch.full((S, P), float("nan"), device=cuda)
        rc = fn(ctypes.byref(ps.desc), ctypes.byref(sd), source_code(st), src.data_ptr(), val.data_ptr(), S,
                N.MODE_RESPONSE, out.data_ptr(), ctypes.byref(o) if o is not None else None, stream)
        assert rc == N.IACT_OK, lib.iact_last_error()
        got = out.double().cpu().numpy()
        assert np.isfinite(got).all()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= IMG_TOL, f"opts {o is not None}: relative L2 {err:.3g} against iact_render"
    out = torch.zeros((S + 1, P), device=cuda)
    rc = fn(ctypes.byref(ps.desc), ctypes.byref(sd), source_code(st), src.data_ptr(), val.data_ptr(), S + 1,
            N.MODE_RESPONSE, out.data_ptr(), None, stream)
    assert rc == N.IACT_E_UNSUPPORTED
    assert float(out.abs().sum()) == 0.0
    del keep
