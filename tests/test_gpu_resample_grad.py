"""Gradients with respect to the primary surface (curvature, conic, aspheric
coefficients) through on-device resampling: DeviceIntegrator draws the
aperture positions and roughness coefficients once; the sample arrays are a
differentiable function of the surface (FP64 torch restatement); the
adjoint kernel returns per-sample sums dL/d(point, normal, 1/weight)
(iact_render_backward g_samples) which RenderFunction maps to the arrays.
Checked against the FP64 autograd twin on the same samples and the GPU's
decisions (the reference differentiates the primary's asphere coefficients
only through resampling), tolerance GRAD_TOL."""
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
    p, n, dl, w = twin.resample_mapping(g2, surf2, raw.points.cpu(), raw.normals.cpu(),
                                        raw.perturbation_delta.cpu(), raw.weights.cpu(), 96)
    p, n, dl, w = p.float(), n.float(), dl.float(), w.float()
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


def test_resampled_step_replays_in_a_cuda_graph(cuda):
    """The resample (iact_sample_facets with the surface read on the device),
    render, adjoint and sampler reverse of one step, captured once in a CUDA
    graph: a replay gives the eager step's surface and tilt gradients (up to
    the summation order of the float atomics)."""
    from iactrace_gb300 import DifferentiableSquareSensor
    g = _dish(1.0 / 30.0, -0.4, [2e-3, -4e-4])
    g = g.replace(**{n: getattr(g, n).to(cuda) for n in ("positions", "offsets", "vertices", "perturbation_scale")})
    rot = g.rotations.clone().to(cuda).requires_grad_(True)
    a1 = torch.tensor([2e-3, -4e-4], device=cuda, requires_grad=True)
    cam = DifferentiableSquareSensor([0, 0, 15.0], [0, 0, 0], 24, 24, (-0.504, 0.504, -0.504, 0.504), sigma=0.5)
    d = torch.tensor([[0.01, -0.02, -1.0], [-0.015, 0.01, -1.0]], device=cuda)
    d = d / d.norm(dim=1, keepdim=True)
    val = torch.tensor([1.0, 0.7], device=cuda)
    gw = torch.randn((24, 24), generator=torch.Generator(device=cuda).manual_seed(2), device=cuda)
    integ = it.DeviceIntegrator(64)

    def step():
        gs = integ.sample_group(g.replace(aspheric=a1, rotations=rot), 17)
        it.render(Telescope([gs], [], [cam]), d, val, "parallel").backward(gw)

    step()
    ref_a, ref_r = a1.grad.clone(), rot.grad.clone()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        step()
    torch.cuda.current_stream().wait_stream(side)
    a1.grad, rot.grad = None, None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    graph.replay()
    torch.cuda.synchronize()
    for name, x, y in (("aspheric", a1.grad, ref_a), ("rotations", rot.grad, ref_r)):
        err = (x - y).norm() / y.norm()
        assert y.norm() > 0 and err < 1e-5, f"{name}: graph replay differs by {err:.3g}"
