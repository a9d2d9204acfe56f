"""Bundle culling of the shadow tests is exact.

The render kernels restrict each warp's primary shadow tests to the
primitives whose bounding volume comes near the warp's bundle of shadow
rays. The output with culling must equal the output with every primitive tested
on every ray (IACT_FLAG_NO_CULL): same shadow masks, same hits. The two runs
may still differ in the last bits, as two runs of either mode do, because
the FP32 shared-memory atomics of different warps land in varying order; a
single flipped shadow decision moves a whole ray value into or out of a
pixel, at least 1e-5 of that pixel's total on these scenes (fewer than 1e5
rays per pixel), so outputs must agree to FLIP_TOL = 1e-6 per pixel
(relative). Scenes cover every primitive kind, point / parallel / extended
sources, images and response matrices, more candidates than one 32-lane
chunk, and the batched kernel.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import _native as N, Telescope, workloads as W
from iactrace_gb300.core import Cylinder, OrientedBox, Sphere, Triangle, group_obstructions
from iactrace_gb300.core.transforms import euler_to_matrix

from test_gpu_forward import check_image

pytestmark = pytest.mark.gpu


def _opts(no_cull: bool):
    o = N.IactOpts()
    o.flags = N.FLAG_NO_CULL if no_cull else 0
    return o


FLIP_TOL = 1e-6


def _close(a, b):
    d = (a.double() - b.double()).abs()
    bad = d > FLIP_TOL * b.double().abs() + 1e-12 * float(b.abs().max())
    return int(bad.sum()), float((d / b.double().abs().clamp_min(1e-30)).max())


def _same(tel, src, val, st, mode="image", seed=0):
    fn = it.render_response_matrix if mode == "response" else it.render
    a = fn(tel, src, val, st, opts=_opts(False), seed=seed)
    b = fn(tel, src, val, st, opts=_opts(True), seed=seed)
    assert float(b.abs().sum()) > 0
    n_bad, worst = _close(a, b)
    assert n_bad == 0, f"culling changed {n_bad} of {a.numel()} outputs (max relative difference {worst:.3g})"
    return a


def lattice_scene(n_cyl=270, n_samples=32, seed=0):
    """A dish under a lattice of thin struts (CT5-like primitive count):
    n_cyl random cylinders between the rim and the camera, plus the camera
    box, spheres, an oriented box and triangles (workloads.strut_lattice)."""
    groups, _ = W.davies_cotton(n_samples=n_samples, seed=seed, obstructions=False)
    return Telescope(groups, group_obstructions(W.strut_lattice(n_cyl, seed)), [W.hex_camera(960)])


def test_cull_exact_plain_and_response(cuda):
    tel, src, val, st = W.plain_forward(n_samples=256, n_sources=16)
    _same(tel, src, val, st)
    tel, src, val, st = W.response_matrix(n_samples=32, n_side=12)
    _same(tel, src, val, st, mode="response")


def test_cull_exact_parallel_and_near_point_sources(cuda):
    tel, src, val, st = W.plain_forward(n_samples=128, n_sources=4)
    g = torch.Generator().manual_seed(3)
    d = torch.randn(24, 3, generator=g) * 0.03
    d[:, 2] = -1.0
    d[0] = torch.tensor([0.0, 0.0, -1.0])  # exactly along the axis
    _same(tel, d, torch.rand(24, generator=g) + 0.5, "parallel")
    near = torch.tensor([[0.0, 0.0, 40.0], [3.0, -2.0, 25.0], [10.0, 5.0, 200.0], [0.5, 0.5, 17.0]])
    _same(tel, near, torch.ones(4), "point")  # sources close to the dish: wide bundles


def test_cull_exact_many_primitives(cuda):
    tel = lattice_scene()
    src = W.point_sources_disk(12, 2.5, 21)
    _same(tel, src, torch.ones(12), "point")
    _same(tel, src[:6], torch.ones(6), "point", mode="response")
    d = torch.tensor([[0.01, 0.02, -1.0], [-0.03, 0.0, -1.0], [0.0, 0.0, -1.0]])
    _same(tel, d / d.norm(dim=1, keepdim=True), torch.ones(3), "parallel")


def test_cull_many_primitives_against_oracle(cuda):
    tel = lattice_scene(n_samples=8)
    src = W.point_sources_disk(4, 2.5, 22)
    cont, raw, stats = check_image(tel, src, torch.ones(4), "point")
    print(f"lattice: cont {cont:.2e} raw {raw:.2e} {stats}")


def test_cull_exact_extended_sources(cuda):
    from iactrace_gb300 import alignment as A
    pb = A.problem(n_facets=61, n_samples=32, n_sources=24, n_pixels=900, device=cuda)
    tel = pb["telescope"]
    obst = group_obstructions([Cylinder([3.0, 0.0, 1.0], [0.5, 0.0, 35.0], 0.05),
                               Sphere([0.0, 1.5, 20.0], 0.5)])
    tel = Telescope(tel.mirror_groups, obst, tel.sensors)
    _same(tel, pb["sources"], pb["values"], "extended", seed=7)


def test_cull_exact_batched(cuda):
    tels, srcs, vals, st = W.ragged_batch(n_instances=5, n_samples=32, seed=9, max_facets=300, min_facets=60,
                                          max_sources=48)
    a = it.BatchRenderer(tels, srcs, vals, st, opts=_opts(False), tune=False)()
    b = it.BatchRenderer(tels, srcs, vals, st, opts=_opts(True), tune=False)()
    for i, (x, y) in enumerate(zip(a, b)):
        assert _close(x, y)[0] == 0, f"job {i}"
