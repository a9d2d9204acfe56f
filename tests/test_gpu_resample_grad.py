"""Gradients with respect to the primary surface (curvature, conic, aspheric
coefficients) through on-device resampling: DeviceIntegrator draws the
aperture positions and roughness coefficients once; the sample arrays are a
differentiable function of the surface (FP64 torch restatement); the
adjoint kernel returns per-sample sums dL/d(point, normal, 1/weight)
(iact_render_backward g_samples) which RenderFunction maps to the arrays.
Checked against the FP64 autograd twin on the same samples and the GPU's
decisions (primary asphere coefficients "only through
resampling"), tolerance GRAD_TOL."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Mirror, Telescope, workloads as W
from iactrace_gb300.core import AsphericSurface, PolygonAperture
from iactrace_gb300.telescope.mirrors import group_mirrors

import twin

GRAD_TOL = 1e-4

pytestmark = pytest.mark.gpu


def _dish(c, k, a):
    surf = AsphericSurface(c, k, a)
    verts = W.hex_vertices(0.6)
    ms = []
    for (x, y) in W.hex_grid(19, 0.62):
        z = 15.0 - (15.0 ** 2 - x * x - y * y) ** 0.5
        ms.append(Mirror([x, y, z], W.dc_orientation((x, y, z), 30.0), surf, PolygonAperture(verts),
                         optical_stage=0))
    return group_mirrors(ms)[0]


def test_resampling_gradients_match_the_twin(cuda):
    from iactrace_gb300 import DifferentiableSquareSensor
    c0, k0, a0 = 1.0 / 30.0, -0.4, [2e-3, -4e-4]
    g = _dish(c0, k0, a0)
    cam = DifferentiableSquareSensor([0, 0, 15.0], [0, 0, 0], 24, 24, (-0.504, 0.504, -0.504, 0.504), sigma=0.5)
    d = torch.tensor([[0.01, -0.02, -1.0], [-0.015, 0.01, -1.0]])
    d = d / d.norm(dim=1, keepdim=True)
    val = torch.tensor([1.0, 0.7])
    gw = np.random.default_rng(5).standard_normal(24 * 24)
    integ = it.DeviceIntegrator(96)
    # GPU: resample with differentiable surface parameters, render, backward
    c1 = torch.tensor(c0, requires_grad=True)
    k1 = torch.tensor(k0, requires_grad=True)
    a1 = torch.tensor(a0, requires_grad=True)
    gs = integ.sample_group(g.replace(curvature=c1, conic=k1, aspheric=a1), 17)
    tel = Telescope([gs], [], [cam])
    img = it.render(tel, d, val, "parallel")
    (img.double().reshape(-1) * torch.as_tensor(gw, device=cuda)).sum().backward()
    # twin: the same drawn samples, the same mapping in FP64 on the CPU
    raw = integ.sample_group(g, 17)  # identical variates, constant surface
    c2 = torch.tensor(c0, dtype=torch.float64, requires_grad=True)
    k2 = torch.tensor(k0, dtype=torch.float64, requires_grad=True)
    a2 = torch.tensor(a0, dtype=torch.float64, requires_grad=True)
    g2 = g.replace(curvature=c2, conic=k2, aspheric=a2)
    surf2 = g2.get_surface()
    p, n, dl, w = integ._differentiable(g2, surf2, raw.points.cpu(), raw.normals.cpu(),
                                        raw.perturbation_delta.cpu(), raw.weights.cpu())
    tel2 = Telescope([g.replace(points=p, normals=n, perturbation_delta=dl, weights=w)], [], [cam])
    pts, vals, pix, _ = it.render_debug(Telescope([raw], [], [cam]), d, val, "parallel", extras=True)
    sc, sn = twin.scene_of(tel2, 0, "parallel")
    dec = {"pix": pix.cpu().numpy(), "alive": vals.cpu().numpy() != 0}
    grp = tel2.mirror_groups[0]
    params = {"rot": grp.rotations.double(), "pos": grp.positions.double(),
              "scale": grp.perturbation_scale.double(), "src": d.double(), "val": val.double(), "mirrors": []}
    out = twin.render(sc, params, dec, sn, "image")
    (out.reshape(-1) * torch.as_tensor(gw)).sum().backward()
    for name, x, y in (("curvature", c1, c2), ("conic", k1, k2), ("aspheric", a1, a2)):
        gx, gy = x.grad.double().cpu().numpy().reshape(-1), y.grad.numpy().reshape(-1)
        err = np.linalg.norm(gx - gy) / np.linalg.norm(gy)
        print(name, gx, gy, err)
        assert np.linalg.norm(gy) > 0
        assert err <= GRAD_TOL, f"d/d{name}: relative error {err:.3g}"
