"""Renders at the maxima the C ABI documents: IACT_MAX_OBSTRUCTIONS (2048)
shadowing primitives of all five kinds and IACT_MAX_STAGE_MIRRORS (64)
stage mirrors, ray by ray against the FP64 oracle (tolerances of
tests/test_gpu_forward.py)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Telescope, _native as N, workloads as W
from iactrace_gb300.core import AsphericSurface, DiskAperture, group_obstructions
from iactrace_gb300.telescope import Mirror, group_mirrors

from test_gpu_forward import check_image

pytestmark = pytest.mark.gpu


def small_primitives(n, seed=2):
    """n small obstructions of all five kinds scattered over and above a
    37-facet dish: thin rods (1600 of 2048), spheres, boxes, oriented boxes
    and triangles, leaving most rays unshadowed."""
    from iactrace_gb300.core import Box, Cylinder, OrientedBox, Sphere, Triangle
    from iactrace_gb300.core.transforms import euler_to_matrix
    rng = np.random.default_rng(seed)
    pt = lambda: [float(rng.uniform(-2.2, 2.2)), float(rng.uniform(-2.2, 2.2)), float(rng.uniform(1.0, 14.0))]
    out = []
    n_obox = n_tri = 24
    n_box, n_sph = 100, 300
    for _ in range(n - n_obox - n_tri - n_box - n_sph):
        a = pt()
        b = [a[0] + float(rng.normal(0, 0.4)), a[1] + float(rng.normal(0, 0.4)), a[2] + float(rng.normal(0, 0.4))]
        out.append(Cylinder(a, b, 0.001))
    for _ in range(n_sph):
        out.append(Sphere(pt(), 0.01))
    for _ in range(n_box):
        c = pt()
        out.append(Box([c[0] - 0.01, c[1] - 0.01, c[2] - 0.01], [c[0] + 0.01, c[1] + 0.01, c[2] + 0.01]))
    for _ in range(n_obox):
        out.append(OrientedBox(pt(), [0.02, 0.01, 0.03], euler_to_matrix(torch.tensor(rng.uniform(0, 90, 3)))))
    for _ in range(n_tri):
        c = pt()
        out.append(Triangle(c, [c[0] + 0.03, c[1], c[2]], [c[0], c[1] + 0.03, c[2] + 0.01]))
    return out


def test_maximum_obstruction_count(cuda):
    """2048 small primitives over a 37-facet dish. Thin rods several metres
    from a ray's origin are at the limit of float32 (|oc|^2 - r^2 with
    r = 1 mm), so some grazing rays flip their shadow decision in any
    float32 evaluation: the GPU's flips against FP64 must be no more than the
    float32 restatement's of the reference chain (+ SLACK); away from shadow
    flips the per-ray pixel ids and values follow the FP64 oracle, culled and
    unculled renders agree, and the adjoint's value gradient is (R g) / v."""
    import oracle.oracle as O
    from test_gpu_forward import EDGE_BAND
    SLACK = 2
    groups, _ = W.davies_cotton(n_facets=37, n_samples=32, seed=1, obstructions=False)
    prims = small_primitives(N.IACT_MAX_OBSTRUCTIONS)
    assert len(prims) == N.IACT_MAX_OBSTRUCTIONS
    tel = Telescope(groups, group_obstructions(prims), [W.hex_camera(960)])
    src, val = W.point_sources_disk(4, 2.5, 3), torch.ones(4)
    pts, vals, pix, _ = it.render_debug(tel, src, val, "point", extras=True)
    g = {"vals": vals.cpu().double().numpy(), "pix": pix.cpu().numpy()}
    o64 = O.render_debug(tel, src, val, "point", 0, "f64")
    o32 = O.render_debug(tel, src, val, "point", 0, "f32")
    flip_gpu = (g["vals"] == 0) != (o64["vals"] == 0)
    flip_32 = (o32["vals"] == 0) != (o64["vals"] == 0)
    print(f"2048 primitives: shadow flips against FP64: GPU {int(flip_gpu.sum())}, float32 restatement "
          f"{int(flip_32.sum())} of {flip_gpu.size} rays; {float((g['vals'] != 0).mean()):.2f} unshadowed")
    assert flip_gpu.sum() <= flip_32.sum() + SLACK
    same = ~flip_gpu & (o64["vals"] != 0)
    bad = same & (g["pix"] != o64["pix"]) & (o64["margin"] >= EDGE_BAND)
    assert not bad.any(), f"{int(bad.sum())} pixel ids differ away from pixel edges"
    verr = np.abs(g["vals"][same] - o64["vals"][same]).max() / np.abs(o64["vals"]).max()
    assert verr < 2e-5
    alive = float((g["vals"] != 0).mean())
    assert 0.05 < alive < 0.95  # the primitives shadow part of the dish
    culled = it.render(tel, src, val, "point").double()
    nc = N.IactOpts()
    nc.flags = N.FLAG_NO_CULL
    every = it.render(tel, src, val, "point", opts=nc).double()
    assert float((culled - every).norm() / every.norm()) < 1e-6
    # the adjoint over the same tables: dL/dv = (R g) / v, R the response matrix
    R = it.render_response_matrix(tel, src, val, "point").double()
    gw = torch.randn(R.shape[1], generator=torch.Generator().manual_seed(0), dtype=torch.float64).to(R.device)
    v = val.clone().cuda().requires_grad_(True)
    (it.render(tel, src, v, "point").double().reshape(-1) * gw).sum().backward()
    want = (R @ gw) / val.double().cuda()
    assert float((v.grad.double() - want).norm() / want.norm()) < 1e-5


def test_maximum_stage_mirror_count(cuda):
    """The Cassegrain's secondary cut into 64 disk segments on one
    hyperboloid: every ray's closest hit is chosen among 64 mirrors."""
    tel, _, _, _ = W.cassegrain(n_samples=16, n_sources=1)
    f = 10.0
    a = 0.5 * ((6.0 + 0.5) - (f - 6.0))
    ch = 0.5 * (f + 0.5)
    sec = AsphericSurface(-a / (ch * ch - a * a), -(ch / a) ** 2, [])
    segs = []
    for i in range(8):
        for j in range(8):
            x0, y0 = -1.05 + 0.3 * i, -1.05 + 0.3 * j
            z0 = float(sec._sag_raw(torch.tensor(x0, dtype=torch.float64), torch.tensor(y0, dtype=torch.float64)))
            segs.append(Mirror([x0, -y0, 6.0 - z0], [180.0, 0.0, 0.0], sec, DiskAperture(0.14), optical_stage=1,
                               offset=[x0, y0]))
    assert len(segs) == N.IACT_MAX_STAGE_MIRRORS
    prim = [g for g in tel.mirror_groups if g.optical_stage == 0]
    tel = Telescope(prim + group_mirrors(segs), [], tel.sensors, name="segmented64")
    th = torch.deg2rad(torch.tensor([0.0, 0.3, 0.5]))
    ph = torch.deg2rad(torch.tensor([0.0, 100.0, 220.0]))
    d = torch.stack([torch.sin(th) * torch.cos(ph), torch.sin(th) * torch.sin(ph), -torch.cos(th)], 1)
    val = torch.tensor([1.0, 0.5, 2.0])
    _, vals, _, hm = it.render_debug(tel, d, val, "parallel", extras=True)
    hit = hm[vals != 0]
    assert hit.numel() > 0.2 * vals.numel() and torch.unique(hit).numel() > 20
    cont, raw, stats = check_image(tel, d, val, "parallel")
    print(f"64 stage mirrors: cont {cont:.2e} raw {raw:.2e} {stats}, {torch.unique(hit).numel()} mirrors hit")
