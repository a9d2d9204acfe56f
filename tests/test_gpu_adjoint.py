"""The adjoint kernel (iact_render_backward behind torch.autograd) against the
torch FP64 autograd twin of the reference chain (tests/twin.py, the stand-in
for jax.grad), on the discrete decisions the GPU took (pixel ids, shadow and
hit masks, soft-splat base pixels: constants under jax.grad).

Tolerance: per parameter block (facet rotations, positions, roughness scales,
sources, values, stage-mirror rotations, positions, surface parameters) the
relative L2 error is <= GRAD_TOL. The twin itself is checked against central
finite differences of the FP64 oracle in tests/test_twin_fd.py.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Telescope, workloads as W

import gradref
import twin

GRAD_TOL = 1e-4

pytestmark = pytest.mark.gpu


def small_dish(camera, seed=2, n_samples=48, roughness=24.0):
    groups, _ = W.davies_cotton(n_facets=19, n_samples=n_samples, seed=seed)
    from iactrace_gb300.core import Box, Cylinder, group_obstructions
    obst = group_obstructions([Cylinder([1.6, 0.4, 0.2], [0.3, 0.1, 15.4], 0.05),
                               Box([-0.3, -0.3, 15.0], [0.3, 0.3, 16.0])])
    tel = Telescope(groups, obst, [camera])
    return tel.apply_roughness(roughness) if roughness else tel


def gpu_grads(tel, src, val, st, g, mode="image"):
    return gradref.gpu_grads(tel, src, val, st, g, mode)


def twin_grads(tel, src, val, st, g, mode="image"):
    """Twin (FP64 autograd) gradients on the GPU's discrete decisions."""
    return gradref.twin_grads(tel, src, val, st, g, gradref.gpu_debug(tel, src, val, st), mode)


def compare(gpu, ref, tol=GRAD_TOL, skip=()):
    return gradref.compare(gpu, ref, tol, skip)


@pytest.mark.parametrize("mode", ["image", "response"])
def test_adjoint_hard_square_point_sources(cuda, mode):
    from iactrace_gb300 import SquareSensor
    tel = small_dish(SquareSensor([0, 0, 15.0], [0, 0, 0], 16, 16, (-0.336, 0.336, -0.336, 0.336)))
    src = torch.tensor([[3.0, -2.0, 2000.0], [-20.0, 10.0, 2000.0], [35.0, 25.0, 2000.0]])
    val = torch.tensor([1.0, 0.7, 1.3])
    g = np.random.default_rng(0).standard_normal((3, 256) if mode == "response" else 256)
    print(mode, compare(gpu_grads(tel, src, val, "point", g, mode), twin_grads(tel, src, val, "point", g, mode)))


def _dirs():
    d = torch.tensor([[0.01, -0.02, -1.0], [-0.03, 0.015, -1.0]])
    return d / d.norm(dim=1, keepdim=True), torch.tensor([1.0, 2.0])


def test_adjoint_hard_hex_parallel_sources(cuda):
    tel = small_dish(W.hex_camera(400, 0.042))
    d, val = _dirs()
    g = np.random.default_rng(1).standard_normal(400)
    print(compare(gpu_grads(tel, d, val, "parallel", g), twin_grads(tel, d, val, "parallel", g)))


@pytest.mark.parametrize("kind", ["square", "hex"])
def test_adjoint_soft_sensors_position_path(cuda, kind):
    from iactrace_gb300 import DifferentiableHexagonalSensor, DifferentiableSquareSensor
    if kind == "square":
        cam = DifferentiableSquareSensor([0, 0, 15.0], [0, 0, 0], 16, 16, (-0.336, 0.336, -0.336, 0.336), sigma=0.4)
        P = 256
    else:
        cam = DifferentiableHexagonalSensor([0, 0, 15.0], [0, 0, 0], W.hex_grid(400, 0.042), sigma=0.35)
        P = 400
    tel = small_dish(cam)
    d, val = _dirs()
    g = np.random.default_rng(2).standard_normal(P)
    # pixels fed by rays on a kink of the hexagonal norm carry no weight:
    # the one-sided derivatives there differ between float32 and float64
    pts, _ = it.render_debug(tel, d, val, "parallel")
    _, sn = twin.scene_of(tel, 0, "parallel")
    kink = twin.soft_hex_kink_pixels(sn, pts.cpu().numpy())
    g[kink] = 0.0
    print(kind, f"{kink.size} kink pixels", compare(gpu_grads(tel, d, val, "parallel", g),
                                                     twin_grads(tel, d, val, "parallel", g)))


def test_adjoint_cassegrain_through_the_secondary(cuda):
    """Gradients through the Newton root of the hyperbolic secondary: primary
    tilts, sources, secondary pose and surface (curvature, conic, aspheric)."""
    tel, src, val, st = W.cassegrain(n_samples=24, n_sources=6)
    sec = [g for g in tel.mirror_groups if g.optical_stage == 1][0]
    tel = Telescope([g if g.optical_stage == 0 else g.replace(aspheric=torch.tensor([1e-4, -2e-6]))
                     for g in tel.mirror_groups], [], tel.sensors)
    del sec
    src = torch.tensor([[30.0, -20.0, 3000.0], [-45.0, 10.0, 3000.0], [5.0, 60.0, 3000.0]])
    val = torch.tensor([1.0, 0.5, 2.0])
    g = np.random.default_rng(3).standard_normal(1024)
    print(compare(gpu_grads(tel, src, val, "point", g), twin_grads(tel, src, val, "point", g)))
