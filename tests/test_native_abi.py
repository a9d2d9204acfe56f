"""The C ABI library: loads without a GPU, exports every declared symbol,
agrees with the binding on struct layouts and validates its arguments."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

from iactrace_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "iactrace_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char\*)\s+(iact_\w+)\s*\(", src, re.M)))


def test_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(N.lib_path())
    syms = declared_symbols()
    assert "iact_render" in syms and "iact_render_debug" in syms and "iact_batch_destroy" in syms
    assert sorted(N.EXPORTED) == [x for x in syms if x != "iact_render_noalloc"]
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/iactrace_gb300.h but not exported"


def test_layout_and_version(built):
    N.check_layout(built)
    assert built.iact_abi_version() == 3


def _square(n=4):
    sn = N.IactSensor()
    sn.type, sn.n_pixels, sn.width, sn.height, sn.dx, sn.dy = N.SENSOR_SQUARE, n * n, n, n, 0.1, 0.1
    return sn


def test_workspace_size_and_validation(built):
    sc, sn = N.IactScene(), _square()
    sz = ctypes.c_size_t(0)
    ws = lambda S, mode: built.iact_workspace_size(ctypes.byref(sc), ctypes.byref(sn), S, mode, ctypes.byref(sz))
    assert ws(0, N.MODE_IMAGE) == 0 and sz.value > 0
    img = sz.value
    assert ws(100, N.MODE_RESPONSE) == 0 and sz.value >= img + 100 * 16 * 8 - 256
    assert ws(3, 7) == N.IACT_E_INVALID
    sc.n_facets, sc.n_samples = 4, 8  # arrays missing
    assert ws(1, N.MODE_IMAGE) == N.IACT_E_INVALID
    assert b"non-NULL" in built.iact_last_error()
    sc = N.IactScene()
    sc.n_cyl = 3  # table missing
    assert ws(1, N.MODE_IMAGE) == N.IACT_E_INVALID


def test_render_rejects_bad_arguments_before_any_cuda_call(built):
    sc, sn = N.IactScene(), N.IactSensor()
    rc = built.iact_render(ctypes.byref(sc), ctypes.byref(sn), 0, None, None, 0, 0, None, None, 0, None, None)
    assert rc == N.IACT_E_INVALID  # sensor without pixels
    sn.type, sn.n_pixels, sn.width, sn.height, sn.dx, sn.dy = N.SENSOR_SQUARE, 4, 2, 2, 0.1, 0.1
    rc = built.iact_render(ctypes.byref(sc), ctypes.byref(sn), 7, None, None, 0, 0, None, None, 0, None, None)
    assert rc == N.IACT_E_INVALID and b"source_type" in built.iact_last_error()
    rc = built.iact_render(ctypes.byref(sc), ctypes.byref(sn), 0, None, None, 0, 0, None, None, 0, None, None)
    assert rc == N.IACT_E_WORKSPACE
    sn.type = N.SENSOR_HEX
    rc = built.iact_render(ctypes.byref(sc), ctypes.byref(sn), 0, None, None, 0, 0, None, None, 0, None, None)
    assert rc == N.IACT_E_INVALID and b"lookup table" in built.iact_last_error()


def test_refused_calls_launch_nothing(built):
    """The launch counter moves only for kernels actually queued: calls
    refused by validation (and, without a GPU, launches that fail) leave
    it where it was."""
    n0 = built.iact_kernel_launches()
    assert n0 >= 0
    sc, sn = N.IactScene(), _square()
    assert built.iact_render(ctypes.byref(sc), ctypes.byref(sn), 7, None, None, 0, 0, None, None, 0, None,
                             None) == N.IACT_E_INVALID
    assert built.iact_probe_fma(None, 1, 1, None) == N.IACT_E_INVALID
    assert built.iact_kernel_launches() == n0


def test_render_without_device_fails_loudly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    import iactrace_gb300 as it
    from iactrace_gb300 import workloads as W
    tel, src, val, st = W.plain_forward(n_samples=4, n_sources=1)
    with pytest.raises(RuntimeError):
        it.render(tel, src, val, st)


def _fake_scene(F, M, n_cyl=0):
    """Descriptor of F facets x M samples with dummy (never dereferenced) device pointers."""
    sc = N.IactScene()
    sc.n_facets, sc.n_samples = F, M
    p = 0x10000
    for name in ("facet_pos", "facet_rot", "facet_scale", "points", "normals", "delta", "weights"):
        setattr(sc, name, p)
    if n_cyl:
        sc.n_cyl, sc.cyl = n_cyl, p
    return sc


def test_batch_planner_without_a_gpu(built):
    """iact_batch_create plans on the host only: tiles, rays, classes and the
    workspace size follow from the jobs; bad arguments are rejected."""
    scenes = [_fake_scene(100, 256, 4), _fake_scene(37, 64), _fake_scene(5, 33)]
    sn = _square(8)
    S = [7, 1, 0]
    jobs = (N.IactJob * 3)()
    for i in range(3):
        jobs[i].scene = ctypes.pointer(scenes[i])
        jobs[i].sensor = ctypes.pointer(sn)
        jobs[i].sources = jobs[i].values = 0x20000 if S[i] else None
        jobs[i].n_sources = S[i]
        jobs[i].out = 0x30000
    h = ctypes.c_void_p()
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, N.MODE_IMAGE, None, ctypes.byref(h)) == N.IACT_OK
    info = (ctypes.c_int64 * 5)()
    assert built.iact_batch_info(h, info, 5) == N.IACT_OK
    assert info[0] == 3 and info[2] == 100 * 256 * 7 + 37 * 64 * 1
    assert info[1] > 0 and info[4] == 1 and info[3] == 3  # prep, one render class, finish
    size = ctypes.c_size_t(0)
    assert built.iact_batch_workspace_size(h, ctypes.byref(size)) == N.IACT_OK
    assert size.value >= (100 * 256 + 37 * 64 + 5 * 33) * 32 + 3 * 64 * 8
    assert built.iact_batch_render(h, None) == N.IACT_E_INVALID  # not prepared: nothing queued
    assert b"prepare" in built.iact_last_error()
    assert built.iact_batch_backward(h, None) == N.IACT_E_INVALID  # created without the backward flag
    built.iact_batch_destroy(h)
    # with the backward plan: every non-empty job needs dL/d(out)
    opts = N.IactOpts()
    opts.flags = N.FLAG_BATCH_BACKWARD
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, N.MODE_IMAGE, ctypes.byref(opts),
                                   ctypes.byref(h)) == N.IACT_E_INVALID
    assert b"grad_out" in built.iact_last_error()
    for i in range(3):
        jobs[i].grad_out = 0x40000
        jobs[i].g_facet_rot = 0x50000
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, N.MODE_IMAGE, ctypes.byref(opts), ctypes.byref(h)) == 0
    info7 = (ctypes.c_int64 * 7)()
    assert built.iact_batch_info(h, info7, 7) == N.IACT_OK
    assert info7[5] > 0 and info7[6] == 3  # prep + one adjoint class + finish
    size_b = ctypes.c_size_t(0)
    assert built.iact_batch_workspace_size(h, ctypes.byref(size_b)) == N.IACT_OK
    assert size_b.value > size.value  # + roughness deltas and gradient buckets
    built.iact_batch_destroy(h)
    for i in range(3):
        jobs[i].grad_out = None
        jobs[i].g_facet_rot = None
    # rejected jobs
    jobs[1].out = None
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, N.MODE_IMAGE, None, ctypes.byref(h)) == N.IACT_E_INVALID
    assert b"job 1" in built.iact_last_error()
    jobs[1].out = 0x30000
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, 9, None, ctypes.byref(h)) == N.IACT_E_INVALID
    opts = N.IactOpts()
    opts.block_threads = 100
    assert built.iact_batch_create(jobs, 3, N.SRC_POINT, N.MODE_IMAGE, ctypes.byref(opts),
                                   ctypes.byref(h)) == N.IACT_E_INVALID
    assert built.iact_batch_create(jobs, -1, N.SRC_POINT, N.MODE_IMAGE, None, ctypes.byref(h)) == N.IACT_E_INVALID


def test_tile_defaults_without_a_gpu(built):
    """Default work-tile sizes of the host planner (read back through the
    batch planner, which plans on the host only), at 256 threads per CTA
    and 100 facets x 256 samples x 64 sources: a hard-pixel response job
    takes tiles of 192 warp tasks per warp (4 sources x 48 facets x 8
    32-sample chunks: 16 x 3 tiles); a soft-pixel response job 48 (4 x 12 x
    8: 16 x 9); an image job 48 (8 x 6 x 8: 8 x 17); an explicit
    opts.tasks_per_warp wins."""
    sc = _fake_scene(100, 256)
    hard = _square(8)
    soft = _square(8)
    soft.type, soft.sigma, soft.kernel_size = N.SENSOR_SOFT_SQUARE, 0.1, 2

    def tiles(sn, mode, tpw=0):
        job = (N.IactJob * 1)()
        job[0].scene, job[0].sensor = ctypes.pointer(sc), ctypes.pointer(sn)
        job[0].sources = job[0].values = 0x20000
        job[0].n_sources = 64
        job[0].out = 0x30000
        opts = N.IactOpts()
        opts.tasks_per_warp = tpw
        h = ctypes.c_void_p()
        rc = built.iact_batch_create(job, 1, N.SRC_POINT, mode, ctypes.byref(opts), ctypes.byref(h))
        assert rc == N.IACT_OK, built.iact_last_error()
        info = (ctypes.c_int64 * 5)()
        assert built.iact_batch_info(h, info, 5) == N.IACT_OK
        built.iact_batch_destroy(h)
        return int(info[1])

    assert tiles(hard, N.MODE_RESPONSE) == 16 * 3
    assert tiles(soft, N.MODE_RESPONSE) == 16 * 9
    assert tiles(hard, N.MODE_IMAGE) == 8 * 17
    assert tiles(hard, N.MODE_RESPONSE, tpw=48) == 16 * 9


def test_size_limits_are_validated(built):
    """The documented maxima pass and one more is refused, before any GPU
    work: IACT_MAX_OBSTRUCTIONS primitives, IACT_MAX_STAGE_MIRRORS stage
    mirrors, 2^30 primary samples."""
    sn, sz = _square(), ctypes.c_size_t(0)

    def ws(sc):
        return built.iact_workspace_size(ctypes.byref(sc), ctypes.byref(sn), 1, N.MODE_IMAGE, ctypes.byref(sz))

    assert ws(_fake_scene(4, 8, n_cyl=N.IACT_MAX_OBSTRUCTIONS)) == N.IACT_OK
    assert ws(_fake_scene(4, 8, n_cyl=N.IACT_MAX_OBSTRUCTIONS + 1)) == N.IACT_E_UNSUPPORTED
    assert b"IACT_MAX_OBSTRUCTIONS" in built.iact_last_error()
    for n, rc in ((N.IACT_MAX_STAGE_MIRRORS, N.IACT_OK), (N.IACT_MAX_STAGE_MIRRORS + 1, N.IACT_E_UNSUPPORTED)):
        sc = _fake_scene(4, 8)
        sc.n_mirrors, sc.n_stages, sc.mirrors = n, 1, 0x10000
        assert ws(sc) == rc, n
    assert ws(_fake_scene(1 << 15, 1 << 15)) == N.IACT_OK
    assert ws(_fake_scene(1 << 15, (1 << 15) + 1)) == N.IACT_E_UNSUPPORTED


def test_pair_mask_workspace_is_capped(built):
    """Renders of scenes with 1..32 primitives keep one candidate word per
    (source, facet) pair in the workspace, up to 2^26 words; beyond that they
    need none (the generic kernel keeps per-tile masks)."""
    from iactrace_gb300 import Telescope, workloads as W
    from iactrace_gb300.core.scene import pack_scene
    tel, _, _, _ = W.plain_forward(n_samples=8, n_sources=1)
    bare = Telescope(tel.mirror_groups, [], tel.sensors)
    F = 380

    def size(t, S):
        ps = pack_scene(t, "cpu")
        sd, keep = t.sensors[0].pack("cpu")
        sz = ctypes.c_size_t(0)
        N.check(built.iact_workspace_size(ctypes.byref(ps.desc), ctypes.byref(sd), S, N.MODE_IMAGE,
                                          ctypes.byref(sz)))
        del keep
        return sz.value

    S = 1000
    assert size(tel, S) - size(bare, S) >= S * F * 4  # facet bounds + the pair words
    S = (1 << 26) // F + 1
    assert size(tel, S) - size(bare, S) < 1000 * F * 4  # facet bounds only
