"""On-device Monte-Carlo facet sampling (iact_sample_facets, DeviceIntegrator).

* replay: the FP64 oracle (oracle_sample_facets) replays the same
  counter-based variates; the device arrays equal it to float32 rounding;
* distribution: the samples follow MCIntegrator's (the reference's)
  distribution: uniform on the disk / polygon, normals of the surface,
  unit-normal roughness coefficients, weights cos_z / area * n_samples;
* use: a render of device-sampled facets agrees with the same render of
  host-sampled facets within Monte-Carlo noise.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Mirror, Telescope, workloads as W
from iactrace_gb300.core import AsphericSurface, DiskAperture, PolygonAperture
from iactrace_gb300.core.integrators import sampler_desc
from iactrace_gb300.telescope.mirrors import group_mirrors




def _groups():
    surf = AsphericSurface(0.05, -1.05, [1e-4, -2e-6])
    disk = [Mirror([x, y, 0.0], [0.0, 0.0, 0.0], surf, DiskAperture(r), optical_stage=0, offset=[x, y])
            for x, y, r in ((0.0, 0.0, 0.6), (1.2, 0.3, 0.5), (-2.0, 1.5, 0.45))]
    hexv = W.hex_vertices(0.9)
    poly = [Mirror([x, y, 0.0], [0.0, 0.0, 0.0], surf, PolygonAperture(hexv), optical_stage=0, offset=[x, y])
            for x, y in W.hex_grid(7, 0.92)]
    return group_mirrors(disk)[0], group_mirrors(poly)[0]


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_device_samples_replay_on_the_oracle(cuda, which):
    import oracle.oracle as O
    g = _groups()[which]
    M = 2048
    dev = it.DeviceIntegrator(M).sample_group(g, 7)
    d, keep = sampler_desc(g, 7, M, "cpu")
    pts, nrm, dlt, wts = O.sample_facets(d, len(g), M)
    del keep
    assert np.abs(dev.points.cpu().double().numpy() - pts).max() < 1e-6
    assert np.abs(dev.normals.cpu().double().numpy() - nrm).max() < 1e-6
    assert np.abs(dev.perturbation_delta.cpu().double().numpy() - dlt).max() < 2e-5  # |delta| up to ~6
    assert np.abs(dev.weights.cpu().double().numpy()[..., 0] / wts - 1).max() < 1e-6


@pytest.mark.gpu
def test_device_samples_distribution(cuda):
    disk, poly = _groups()
    M = 20000
    d = it.DeviceIntegrator(M).sample_group(disk, 11)
    xy = d.points[..., :2].cpu().double().numpy()
    for f, R in enumerate((0.6, 0.5, 0.45)):
        r2 = (xy[f] ** 2).sum(-1) / R ** 2
        assert r2.max() <= 1.0 + 1e-6
        assert abs(r2.mean() - 0.5) < 0.01  # uniform on the disk: E[r^2] = R^2 / 2
        ang = np.arctan2(xy[f, :, 1], xy[f, :, 0])
        hist = np.histogram(ang, bins=8, range=(-math.pi, math.pi))[0] / M
        assert np.abs(hist - 1 / 8).max() < 0.01
    dl = d.perturbation_delta.cpu().double().numpy().reshape(-1, 3)
    n = d.normals.cpu().double().numpy().reshape(-1, 3)
    assert np.abs((dl * n).sum(-1)).max() < 1e-5  # tangent to the surface
    th2 = (dl ** 2).sum(-1)  # theta1^2 + theta2^2 ~ chi2(2): mean 2
    assert abs(th2.mean() - 2.0) < 0.05
    # weights: cos_z / (pi R^2) * M, so sum over a facet's samples of 1/w * n_z = area
    w = d.weights.cpu().double().numpy()[..., 0]
    for f, R in enumerate((0.6, 0.5, 0.45)):
        assert np.allclose(n.reshape(3, M, 3)[f, :, 2] / w[f] * M, math.pi * R ** 2, rtol=1e-6)
    # polygon: uniform over the hexagon (each of the 4 fan triangles gets its area share)
    p = it.DeviceIntegrator(M).sample_group(poly, 12)
    xy = p.points[0, :, :2].cpu().double().numpy()
    v = np.array(W.hex_vertices(0.9))
    cnt = np.zeros(4)
    for t in range(4):
        a, b, c = v[0], v[t + 1], v[t + 2]
        den = (b[1] - c[1]) * (a[0] - c[0]) + (c[0] - b[0]) * (a[1] - c[1])
        l1 = ((b[1] - c[1]) * (xy[:, 0] - c[0]) + (c[0] - b[0]) * (xy[:, 1] - c[1])) / den
        l2 = ((c[1] - a[1]) * (xy[:, 0] - c[0]) + (a[0] - c[0]) * (xy[:, 1] - c[1])) / den
        cnt[t] = ((l1 >= -1e-9) & (l2 >= -1e-9) & (1 - l1 - l2 >= -1e-9)).sum()
    assert cnt.sum() >= M - 5
    assert np.allclose(cnt / M, [1 / 6, 1 / 3, 1 / 3, 1 / 6], atol=0.012)


@pytest.mark.gpu
def test_render_with_device_sampled_facets(cuda):
    groups, obst = W.davies_cotton(n_samples=4, seed=3)
    g = groups[0]
    host = it.MCIntegrator(512).sample_group(g, 5)
    devg = it.DeviceIntegrator(512).sample_group(g, 5)
    cam = W.hex_camera(960)
    src = W.point_sources_disk(8, 2.0, 4)
    val = torch.ones(8)
    a = it.render(Telescope([host], obst, [cam]), src, val, "point").double()
    b = it.render(Telescope([devg], obst, [cam]), src, val, "point").double()
    # same total flux and image within Monte-Carlo noise (2 x 194560 rays per image)
    assert abs(float(a.sum() / b.sum()) - 1) < 0.01
    assert float((a - b).norm() / a.norm()) < 0.05


@pytest.mark.parametrize("which", [0, 1])
def test_oracle_sampler_distribution_on_cpu(built, which):
    """The oracle itself (CPU replay) follows the integrator's distribution."""
    import oracle.oracle as O
    g = _groups()[which]
    M = 20000
    d, keep = sampler_desc(g, 3, M, "cpu")
    pts, nrm, dlt, wts = O.sample_facets(d, len(g), M)
    del keep
    # the surface: z = sag(x + ox, y + oy) - sag(ox, oy), normal ~ (-dz/dx, -dz/dy, 1)
    surf = g.get_surface()
    off = g.offsets.double().numpy()
    for f in range(len(g)):
        x = torch.as_tensor(pts[f, :50, 0]); y = torch.as_tensor(pts[f, :50, 1])
        z = surf.sag(x, y, torch.as_tensor(off[f])).numpy()
        assert np.abs(z - pts[f, :50, 2]).max() < 1e-9  # descriptor carries float32 surface constants
    assert np.abs(np.linalg.norm(nrm, axis=-1) - 1).max() < 1e-12
    assert abs((dlt ** 2).sum(-1).mean() - 2.0) < 0.05
    if which == 0:
        r2 = (pts[0, :, :2] ** 2).sum(-1) / 0.6 ** 2
        assert abs(r2.mean() - 0.5) < 0.01 and r2.max() <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_sampler_reverse_matches_the_fp64_mapping(cuda, which):
    """iact_sample_facets_backward against torch FP64 autograd of the same
    mapping (tests/twin.py resample_mapping) on the same drawn samples, for
    random dL/d(points, normals, deltas, weights); and the forward with the
    surface read from device memory equals the by-value forward."""
    import twin
    g = _groups()[which]
    M = 512
    integ = it.DeviceIntegrator(M)
    raw = integ.sample_group(g, 5)
    c = torch.tensor(0.05, device=cuda, requires_grad=True)
    k = torch.tensor(-1.05, device=cuda, requires_grad=True)
    a = torch.tensor([1e-4, -2e-6], device=cuda, requires_grad=True)
    gs = integ.sample_group(g.replace(curvature=c, conic=k, aspheric=a), 5)
    for x, y in ((gs.points, raw.points), (gs.normals, raw.normals), (gs.perturbation_delta, raw.perturbation_delta),
                 (gs.weights, raw.weights)):
        assert torch.equal(x.detach(), y)
    gen = torch.Generator(device="cpu").manual_seed(3 + which)
    G = [torch.randn(t.shape, generator=gen, dtype=torch.float64) for t in (gs.points, gs.normals,
                                                                           gs.perturbation_delta, gs.weights)]
    loss = sum((t.double() * u.to(cuda)).sum() for t, u in zip((gs.points, gs.normals, gs.perturbation_delta,
                                                               gs.weights), G))
    loss.backward()
    c2 = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    k2 = torch.tensor(-1.05, dtype=torch.float64, requires_grad=True)
    a2 = torch.tensor([1e-4, -2e-6], dtype=torch.float64, requires_grad=True)
    g2 = g.replace(curvature=c2, conic=k2, aspheric=a2)
    p, n, dl, w = twin.resample_mapping(g2, g2.get_surface(), raw.points.cpu(), raw.normals.cpu(),
                                        raw.perturbation_delta.cpu(), raw.weights.cpu(), M)
    sum((t * u).sum() for t, u in zip((p, n, dl, w), G)).backward()
    for name, x, y in (("curvature", c, c2), ("conic", k, k2), ("aspheric", a, a2)):
        gx = x.grad.double().cpu().numpy().reshape(-1)
        gy = y.grad.numpy().reshape(-1)
        err = np.abs(gx - gy).max() / np.abs(gy).max()
        assert err < 1e-5, f"d/d{name}: {gx} vs {gy} ({err:.3g})"


@pytest.mark.parametrize("which", [0, 1])
def test_fp64_mapping_matches_oracle_finite_differences(built, which):
    """The torch FP64 mapping that checks the device sampler's reverse
    (tests/twin.py resample_mapping) against central finite differences of
    the oracle's own sampler (same variates, perturbed surface constants):
    d/d(curvature, conic, aspheric) of sum(G * (points, normals, deltas,
    weights)) for random G."""
    import oracle.oracle as O
    import twin
    g = _groups()[which]
    M = 64
    theta0 = [np.float32(0.05), np.float32(-1.05), np.float32(1e-4), np.float32(-2e-6)]
    rng = np.random.default_rng(11 + which)
    G = [rng.standard_normal((len(g), M, 3)) for _ in range(3)] + [rng.standard_normal((len(g), M))]

    def arrays(theta):
        d, keep = sampler_desc(g, 9, M, "cpu")
        d.curvature, d.conic = float(theta[0]), float(theta[1])
        d.n_asph = 2
        d.asph[0], d.asph[1] = float(theta[2]), float(theta[3])
        out = O.sample_facets(d, len(g), M)
        del keep
        return out

    def loss(theta):
        return sum(float((a * b).sum()) for a, b in zip(arrays(theta), G))

    fd = []
    for j in range(4):
        h = abs(float(theta0[j])) * 1e-3
        tp, tm = list(theta0), list(theta0)
        tp[j] = np.float32(float(theta0[j]) + h)
        tm[j] = np.float32(float(theta0[j]) - h)
        fd.append((loss(tp) - loss(tm)) / (float(tp[j]) - float(tm[j])))
    pts, nrm, dlt, wts = arrays(theta0)
    c = torch.tensor(float(theta0[0]), dtype=torch.float64, requires_grad=True)
    k = torch.tensor(float(theta0[1]), dtype=torch.float64, requires_grad=True)
    a = torch.tensor([float(theta0[2]), float(theta0[3])], dtype=torch.float64, requires_grad=True)
    g2 = g.replace(curvature=c, conic=k, aspheric=a)
    p, n, dl, w = twin.resample_mapping(g2, g2.get_surface(), torch.from_numpy(pts), torch.from_numpy(nrm),
                                        torch.from_numpy(dlt), torch.from_numpy(wts)[..., None], M)
    L = sum((t * torch.from_numpy(u).reshape(t.shape)).sum() for t, u in zip((p, n, dl, w), G))
    L.backward()
    ad = [float(c.grad), float(k.grad), float(a.grad[0]), float(a.grad[1])]
    for j, name in enumerate(("curvature", "conic", "a0", "a1")):  # measured: below 1.1e-7 relative
        assert abs(ad[j] - fd[j]) <= 1e-6 * abs(fd[j]), f"d/d{name}: autograd {ad[j]} vs FD {fd[j]}"
