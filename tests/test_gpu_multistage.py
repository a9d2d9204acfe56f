"""Scenes with three and four mirror stages after the primary
(core/render.py:145-149 loops over any number of stages): the forward
against the FP64 oracle, and the adjoint (iact_render_backward) against the
torch FP64 twin on the GPU's decisions, with gradients for every stage
mirror's pose, curvature, conic and aspheric terms.

The adjoint keeps the last two stage reflections of a ray and re-traces
earlier ones from the primary during its reverse sweep, so three stages
re-trace one and four stages re-trace two.

Tolerances: hard pixels: per block relative L2 <= GRAD_TOL (1e-4). Soft
pixels add the sensor-plane position path, where float32 rounding of the
hit (~2e-6 m against a 10 mm splat) is the limit: per block <= GRAD_TOL or
<= 1.5 x the error of the same chain differentiated in float32.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import DifferentiableSquareSensor, SquareSensor, Telescope, workloads as W
from iactrace_gb300.core import AsphericSurface, DiskAperture
from iactrace_gb300.telescope import Mirror, group_mirrors

import gradref
from test_gpu_forward import check_image

GRAD_TOL = 1e-4

pytestmark = pytest.mark.gpu


def many_mirror(n_later, soft=False, n_samples=24):
    """The two-mirror Cassegrain workload with further folding mirrors:
    stage 2 a weakly curved aspheric tertiary folding the beam up (focus near
    z = 1.5), stage 3 a quaternary folding it down (focus near z = 0.9) and,
    for four later stages, stage 4 a weak aspheric folding it up once more
    (focus near z = 1.1). n_later: stages after the primary (3 or 4)."""
    tel, _, _, _ = W.cassegrain(n_samples=n_samples, n_sources=1)
    extra = [Mirror([0.02, -0.01, 0.5], [0.05, -0.04, 0.0], AsphericSurface(0.01, 0.0, [2e-3]), DiskAperture(0.35),
                    optical_stage=2),
             Mirror([0.0, 0.01, 1.2], [180.0, 0.03, 0.0], AsphericSurface(-0.01, -0.5, []), DiskAperture(0.3),
                    optical_stage=3)]
    z_cam = 0.9
    if n_later == 4:
        extra.append(Mirror([0.01, 0.0, 1.0], [0.02, 0.0, 0.0], AsphericSurface(0.005, 0.0, [1e-3]),
                            DiskAperture(0.3), optical_stage=4))
        z_cam = 1.1
    groups = list(tel.mirror_groups) + group_mirrors(extra)
    b = (-0.32, 0.32, -0.32, 0.32)
    cam = DifferentiableSquareSensor([0, 0, z_cam], [0, 0, 0], 32, 32, b, sigma=0.5) if soft else \
        SquareSensor([0, 0, z_cam], [0, 0, 0], 32, 32, b)
    tel = Telescope(groups, [], [cam], name=f"{n_later + 1}-mirror")
    assert len(tel.mirror_groups) == n_later + 1
    src = torch.tensor([[30.0, -20.0, 3000.0], [-45.0, 10.0, 3000.0], [5.0, 25.0, 3000.0]])
    return tel, src, torch.tensor([1.0, 0.5, 2.0]), "point"


@pytest.mark.parametrize("n_later", [3, 4])
def test_forward_many_stages(cuda, n_later):
    tel, src, val, st = many_mirror(n_later)
    cont, raw, stats = check_image(tel, src, val, st)
    _, vals = it.render_debug(tel, src, val, st)
    alive = float((vals != 0).float().mean())
    assert alive > 0.3, f"only {alive:.2f} of the rays reach the camera through every stage"
    print(f"{n_later} stages: cont {cont:.2e} raw {raw:.2e} {stats}, {alive:.2f} of the rays alive")


@pytest.mark.parametrize("n_later", [3, 4])
@pytest.mark.parametrize("mode", ["image", "response"])
def test_adjoint_many_stages_hard(cuda, n_later, mode):
    tel, src, val, st = many_mirror(n_later)
    P = 1024
    g = np.random.default_rng(n_later).standard_normal((3, P) if mode == "response" else P)
    got = gradref.gpu_grads(tel, src, val, st, g, mode)
    want = gradref.twin_grads(tel, src, val, st, g, gradref.gpu_debug(tel, src, val, st), mode)
    assert {f"mc{i}" for i in range(n_later)} <= set(got)
    print(n_later, mode, gradref.compare(got, want, GRAD_TOL))


@pytest.mark.parametrize("n_later", [3, 4])
def test_adjoint_many_stages_soft(cuda, n_later):
    tel, src, val, st = many_mirror(n_later, soft=True)
    g = np.random.default_rng(10 + n_later).standard_normal(1024)
    dbg = gradref.gpu_debug(tel, src, val, st)
    got = gradref.gpu_grads(tel, src, val, st, g)
    want = gradref.twin_grads(tel, src, val, st, g, dbg)
    tw32 = gradref.twin_grads(tel, src, val, st, g, dbg, dtype=torch.float32)
    rel = lambda a, b: float(np.linalg.norm(np.reshape(a, -1) - np.reshape(b, -1)) / np.linalg.norm(b))
    errs = {k: (rel(got[k], want[k]), rel(tw32[k], want[k])) for k in want if np.linalg.norm(want[k]) > 0}
    print(n_later, "soft GPU / float32 chain:", {k: f"{a:.2e} / {b:.2e}" for k, (a, b) in errs.items()})
    bad = {k: v for k, v in errs.items() if v[0] > max(GRAD_TOL, 1.5 * v[1])}
    assert not bad, bad
