"""The specialised kernels equal the generic ones.

Renders of single-stage scenes with at most 32 shadowing primitives and an
axis-aligned sensor run k_render_hard (hard pixels) or k_render_soft (soft
pixels, also extended sources), with candidate words per (source, facet)
pair from k_masks; their adjoints k_adjoint_hard / k_adjoint_soft; batch
classes whose jobs all qualify the batched hard-pixel forms; soft-pixel
images of at least 32 sources k_render_soft_spread (one source per lane).
Everything else runs the generic kernels. Both evaluate the same per-ray
arithmetic, so on the same scene they must give the same outputs up to the
order of the sums: the generic
kernel is forced here by options the hard path does not take (histogram
rows in the FP64 accumulator; roughness-scale gradients), and images,
response matrices and gradients are compared at SUM_TOL (relative, per
entry for outputs; per parameter block, relative L2, for gradients).
"""
from __future__ import annotations

import ctypes

import pytest
import torch

import numpy as np

import iactrace_gb300 as it
from iactrace_gb300 import _native as N, Telescope, alignment as A, workloads as W
from iactrace_gb300.sensors import DifferentiableHexagonalSensor, DifferentiableSquareSensor
from iactrace_gb300.core.render import source_code
from iactrace_gb300.core.scene import pack_scene

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6  # FP32 shared-memory rows vs direct FP64 adds: summation order only


def _generic_opts():
    o = N.IactOpts()
    o.hist_mode = 2  # histogram in the FP64 accumulator: not a hard-kernel launch
    return o


def _scenes():
    plain = W.plain_forward(n_samples=96, n_sources=6)  # square camera, 4 masts + camera box
    resp = W.response_matrix(n_samples=64, n_side=6)  # 2048-pixel hexagonal camera
    tel, src, val, _ = resp
    bare = (Telescope(tel.mirror_groups, [], tel.sensors), src, val, "point")  # no primitives
    par = (tel, -src / src.norm(dim=1, keepdim=True), val, "parallel")
    soft_sq = DifferentiableSquareSensor([0.0, 0.0, 15.0], [0.0, 0.0, 0.0], 32, 30, (-0.672, 0.672, -0.63, 0.63),
                                         sigma=0.5, kernel_size=2)
    soft_hx = DifferentiableHexagonalSensor([0.0, 0.0, 15.0], [0.0, 0.0, 0.0],
                                            W.hex_grid(2048, 0.042).astype(np.float32), sigma=0.5, kernel_size=1)
    ptel, psrc, pval, _ = plain
    ext = A.extended_sources(8, max_deg=2.0, seed=7)
    # image renders of >= 32 sources take the source-per-lane soft body:
    # 48 sources (a second, half-filled 32-source block) under the masts, 64
    # extended sources
    _, src48, val48, _ = W.plain_forward(n_samples=96, n_sources=48)
    ext64 = A.extended_sources(64, max_deg=2.0, seed=9)
    return {"plain": plain, "response_hex": resp, "no_obstructions": bare, "parallel": par,
            "soft_square": (Telescope(ptel.mirror_groups, ptel.obstruction_groups, [soft_sq]), psrc, pval, "point"),
            "soft_hex_extended": (Telescope(tel.mirror_groups, tel.obstruction_groups, [soft_hx]), ext,
                                  torch.ones(8), "extended"),
            "soft_square_48": (Telescope(ptel.mirror_groups, ptel.obstruction_groups, [soft_sq]), src48, val48,
                               "point"),
            "soft_hex_extended_64": (Telescope(tel.mirror_groups, tel.obstruction_groups, [soft_hx]), ext64,
                                     torch.rand(64, generator=torch.Generator().manual_seed(4)) + 0.5, "extended")}


SCENES = ["plain", "response_hex", "no_obstructions", "parallel", "soft_square", "soft_hex_extended",
          "soft_square_48", "soft_hex_extended_64"]


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("mode", ["image", "response"])
def test_hard_render_equals_generic(cuda, name, mode):
    tel, src, val, st = _scenes()[name]
    src, val = src.to(cuda), val.to(cuda)
    fn = it.render_response_matrix if mode == "response" else it.render
    a = fn(tel, src, val, st, seed=11).double()
    b = fn(tel, src, val, st, opts=_generic_opts(), seed=11).double()
    assert float(b.abs().sum()) > 0
    bad = (a - b).abs() > SUM_TOL * b.abs() + 1e-12 * float(b.abs().max())
    assert int(bad.sum()) == 0, f"{int(bad.sum())} of {b.numel()} entries differ beyond {SUM_TOL}"


def _backward(lib, ps, sd, code, src, val, mode, gout, scale, seed=0):
    """iact_render_backward through the C ABI: facet rotations and positions,
    sources, values; with `scale` also the roughness scales (which the hard
    adjoint does not take, so the generic kernel runs)."""
    dev = src.device
    S = src.shape[0]
    ws = torch.empty(ps.workspace_bytes(sd, S, N.MODE_BACKWARD), dtype=torch.uint8, device=dev)
    g = [torch.zeros((ps.F, 3), device=dev), torch.zeros((ps.F, 3), device=dev), torch.zeros(ps.F, device=dev),
         torch.zeros((S, 3), device=dev), torch.zeros(S, device=dev)]
    ext = code == N.SRC_EXTENDED  # no source gradients for extended sources
    opts = N.IactOpts()
    opts.seed = seed
    N.check(lib.iact_render_backward(ctypes.byref(ps.desc), ctypes.byref(sd), code, src.data_ptr(), val.data_ptr(),
                                     S, mode, gout.data_ptr(), g[0].data_ptr(), g[1].data_ptr(),
                                     g[2].data_ptr() if scale else None, None if ext else g[3].data_ptr(),
                                     g[4].data_ptr(), None, None, None, None, ws.data_ptr(), ws.numel(),
                                     ctypes.byref(opts), torch.cuda.current_stream(dev).cuda_stream))
    out = {"rot": g[0], "pos": g[1], "val": g[4]}
    if not ext:
        out["src"] = g[3]
    return out


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("mode", ["image", "response"])
def test_hard_adjoint_equals_generic(cuda, name, mode):
    tel, src, val, st = _scenes()[name]
    src, val = src.to(cuda).contiguous(), val.to(cuda).contiguous()
    lib = N.load()
    ps = pack_scene(tel, cuda)
    sd, keep = tel.sensors[0].pack(cuda)
    fn = it.render_response_matrix if mode == "response" else it.render
    out = fn(tel, src, val, st, seed=11)
    gout = torch.randn(out.shape, device=cuda, generator=torch.Generator(device=cuda).manual_seed(3)).contiguous()
    nm = N.MODE_RESPONSE if mode == "response" else N.MODE_IMAGE
    hard = _backward(lib, ps, sd, source_code(st), src, val, nm, gout, scale=False, seed=11)
    generic = _backward(lib, ps, sd, source_code(st), src, val, nm, gout, scale=True, seed=11)
    for k in hard:
        a, b = hard[k].double(), generic[k].double()
        nb = float(b.norm())
        if nb == 0:  # e.g. facet positions under parallel sources and hard pixels: no path carries gradient
            assert float(a.abs().max()) == 0, k
            continue
        err = float((a - b).norm()) / nb
        assert err <= 1e-5, f"{k}: relative L2 {err:.3g} between the hard and the generic adjoint"
    del keep


def test_batched_hard_classes_equal_generic(cuda):
    """A batch whose class runs k_batch_render_hard / k_batch_adjoint_hard
    against the same jobs forced onto the generic batched kernels (global
    histogram rows; roughness-scale gradients requested)."""
    tels, srcs, vals, st = W.ragged_batch(n_instances=6, n_samples=32, max_sources=48, max_facets=300)
    srcs = [s.to(cuda) for s in srcs]
    vals = [v.to(cuda) for v in vals]
    gen = torch.Generator(device=cuda).manual_seed(5)
    hard = it.BatchRenderer(tels, srcs, vals, st, tune=False, graph=False, backward=True,
                            grads=("rot", "pos", "src", "val"))
    generic = it.BatchRenderer(tels, srcs, vals, st, tune=False, graph=False, backward=True, opts=_generic_opts(),
                               grads=("rot", "pos", "scale", "src", "val"))
    for a, b in zip(hard.grad_outs, generic.grad_outs):
        g = torch.randn(a.shape, device=cuda, generator=gen)
        a.copy_(g)
        b.copy_(g)
    oa, ob = hard(), generic()
    for x, y in zip(oa, ob):
        x, y = x.double(), y.double()
        bad = (x - y).abs() > SUM_TOL * y.abs() + 1e-12 * float(y.abs().max())
        assert int(bad.sum()) == 0
    ga, gb = hard.backward(), generic.backward()
    for da, db in zip(ga, gb):
        for k in ("rot", "pos", "src", "val"):
            nb = float(db[k].double().norm())
            if nb == 0:
                assert float(da[k].abs().max()) == 0
                continue
            err = float((da[k].double() - db[k].double()).norm()) / nb
            assert err <= 1e-5, f"{k}: relative L2 {err:.3g}"


def test_render_beyond_the_pair_word_cap(cuda):
    """An image render of more than 2^26 (source, facet) pairs keeps per-tile
    masks (generic kernel); it equals the sum of the same render split into
    two halves of the sources, each of which takes the pair words."""
    tel, _, _, st = W.plain_forward(n_samples=1, n_sources=1)
    F = 380
    S = (1 << 26) // F + 64
    src = W.point_sources_disk(S, 2.5, 9).to(cuda)
    val = (0.5 + torch.rand(S, generator=torch.Generator().manual_seed(10))).to(cuda)
    whole = it.render(tel, src, val, st).double()
    h = S // 2
    halves = (it.render(tel, src[:h], val[:h], st).double() + it.render(tel, src[h:], val[h:], st).double())
    assert float(whole.abs().sum()) > 0
    err = float((whole - halves).norm() / halves.norm())
    assert err <= 1e-6, f"relative L2 {err:.3g} between the capped render and its halves"
