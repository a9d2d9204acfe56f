"""Monte-Carlo facet sampling (core/integrators.py of the reference).

``MCIntegrator.sample_group`` fills a stage-0 mirror group with local sample
points, unit normals, unit-sigma roughness deltas and weights
``cos_z / area * n_samples`` (core/integrators.py:97-187), on the host.
``DeviceIntegrator`` draws the same distribution on the GPU
(``iact_sample_facets``): counter-based Philox variates keyed by (seed,
facet, sample), FP64 arithmetic, float32 arrays left on the device.
"""
from __future__ import annotations

import ctypes
import math
from abc import ABC, abstractmethod

import torch

from .. import _native as N
from ..utils import keys as _keys
from ..utils.sampling import sample_disk, sample_polygon
from .reflection import compute_perturbation_delta


class Integrator(ABC):
    """core/integrators.py:18-55."""

    @abstractmethod
    def sample_group(self, group, key):
        ...

    def sample_mirror_groups(self, mirror_groups, key):
        if not mirror_groups:
            return []
        ks = _keys.split(key, len(mirror_groups) + 1)
        return [self.sample_group(g, k) for g, k in zip(mirror_groups, ks[:-1])]


class MCIntegrator(Integrator):
    """core/integrators.py:58-95."""

    def __init__(self, n_samples: int = 128):
        self.n_samples = int(n_samples)

    def sample_group(self, group, key):
        params = group.get_sampling_params()
        if params["type"] == "disk":
            return self._sample_disk_group(group, key, params)
        if params["type"] == "polygon":
            return self._sample_polygon_group(group, key, params)
        raise TypeError(f"Unknown MirrorGroup type: {params['type']}")

    def _finish(self, group, surface, xy, offsets, area, gen):
        # core/integrators.py:119-127 / 165-175
        pts, nrm = surface.point_and_normal(xy, offsets[:, None, :])
        delta = compute_perturbation_delta(nrm, gen)
        w = nrm[..., 2:3] / area[:, None, None] * self.n_samples
        return group.with_samples(pts.float(), nrm.float(), delta.float(), w.float())

    def _sample_disk_group(self, group, key, params):
        """core/integrators.py:97-140."""
        gen = _keys.generator(key)
        n = len(group)
        radii = params["radii"].double()
        xy = sample_disk(gen, (n, self.n_samples), dtype=torch.float64) * radii[:, None, None]
        area = math.pi * radii ** 2
        return self._finish(group, params["surface"], xy, params["offsets"].double(), area, gen)

    def _sample_polygon_group(self, group, key, params):
        """core/integrators.py:142-187."""
        gen = _keys.generator(key)
        verts = params["vertices"].double()
        xy = torch.stack([sample_polygon(gen, v, (self.n_samples,), dtype=torch.float64) for v in verts])
        x, y = verts[..., 0], verts[..., 1]
        area = 0.5 * torch.abs(torch.sum(x * torch.roll(y, -1, -1) - torch.roll(x, -1, -1) * y, -1))
        return self._finish(group, params["surface"], xy, params["offsets"].double(), area, gen)


def sampler_desc(group, key, n_samples: int, device, surface=None):
    """The iact_sampler_t of a stage-0 group and its arrays on `device`
    (returns the descriptor and the tensors it points at). surface: an
    optional device float32 tensor [2 + n_asph] (curvature, conic,
    aspheric) read by the kernels instead of the group's values; the host
    then reads no parameter value (a captured launch follows updates)."""
    params = group.get_sampling_params()
    surf = params["surface"]
    d = N.IactSampler()
    d.n_facets, d.n_samples = len(group), int(n_samples)
    n_asph = int(torch.as_tensor(surf.aspheric).numel()) if surface is None else int(surface.numel()) - 2
    if n_asph > N.IACT_MAX_ASPH:
        raise ValueError(f"at most {N.IACT_MAX_ASPH} aspheric coefficients")
    d.n_asph = n_asph
    if surface is None:
        value = lambda x: float(x.detach()) if isinstance(x, torch.Tensor) else float(x)
        d.curvature, d.conic = value(surf.curvature), value(surf.conic)
        for i, v in enumerate(torch.as_tensor(surf.aspheric).detach().reshape(-1).tolist()):
            d.asph[i] = float(v)
        keep = []
    else:
        keep = [surface]
        d.surface = surface.data_ptr()
    keep.append(params["offsets"].reshape(-1, 2).to(device=device, dtype=torch.float32).contiguous())
    d.offsets = keep[-1].data_ptr()
    if params["type"] == "disk":
        d.aperture = N.APERTURE_DISK
        keep.append(params["radii"].reshape(-1).to(device=device, dtype=torch.float32).contiguous())
        d.radii = keep[-1].data_ptr()
    else:
        d.aperture = N.APERTURE_POLYGON
        v = params["vertices"].to(device=device, dtype=torch.float32).contiguous()
        if v.shape[1] > N.IACT_MAX_POLY:
            raise ValueError(f"polygon apertures have at most {N.IACT_MAX_POLY} vertices")
        d.n_vert = int(v.shape[1])
        keep.append(v)
        d.vertices = v.data_ptr()
    d.seed = _keys.as_key(key).value & 0xFFFFFFFF
    return d, keep


def _launch_sample(d, F, M, dev):
    pts, nrm, dlt = (torch.empty((F, M, 3), device=dev) for _ in range(3))
    w = torch.empty((F, M, 1), device=dev)
    N.check(N.load().iact_sample_facets(ctypes.byref(d), pts.data_ptr(), nrm.data_ptr(), dlt.data_ptr(),
                                        w.data_ptr(), torch.cuda.current_stream(dev).cuda_stream))
    return pts, nrm, dlt, w


class _SampleFunction(torch.autograd.Function):
    """Sample arrays as a function of the surface vector theta = (curvature,
    conic, aspheric...): iact_sample_facets forward, its reverse
    iact_sample_facets_backward (dL/d theta from dL/d(points, normals,
    deltas, weights)) backward."""

    @staticmethod
    def forward(ctx, theta, desc, keep, F, M):
        ctx.desc, ctx.keep = desc, keep
        ctx.save_for_backward(theta)
        return _launch_sample(desc, F, M, theta.device)

    @staticmethod
    def backward(ctx, gp, gn, gd, gw):
        (theta,) = ctx.saved_tensors
        dev = theta.device
        g = torch.empty(theta.numel(), dtype=torch.float64, device=dev)
        ptr = lambda t: t.contiguous().data_ptr() if t is not None else None
        gs = [t.contiguous() if t is not None else None for t in (gp, gn, gd, gw)]
        N.check(N.load().iact_sample_facets_backward(ctypes.byref(ctx.desc), *(ptr(t) for t in gs), g.data_ptr(),
                                                     torch.cuda.current_stream(dev).cuda_stream))
        return g.to(theta.dtype), None, None, None, None


class DeviceIntegrator(Integrator):
    """MCIntegrator on the GPU: same aperture, surface, roughness-delta and
    weight construction (core/integrators.py:97-187), variates from the
    counter-based stream of iact_sample_facets (reproducible on any host)."""

    def __init__(self, n_samples: int = 128, device=None):
        self.n_samples = int(n_samples)
        self.device = device

    def sample_group(self, group, key):
        """Sample `group` on the device. When the surface parameters
        (curvature, conic, aspheric) are autograd tensors, the arrays are a
        differentiable function of them (resampling gradients through
        iact_sample_facets_backward); the kernels then read the parameters
        from device memory (keep them on the device to capture a step in a
        CUDA graph)."""
        dev = torch.device(self.device) if self.device is not None else torch.device("cuda", torch.cuda.current_device())
        F, M = len(group), self.n_samples
        surf = group.get_surface()
        params = [surf.curvature, surf.conic, surf.aspheric]
        grad = any(isinstance(t, torch.Tensor) and t.requires_grad for t in params)
        on_dev = any(isinstance(t, torch.Tensor) and t.is_cuda for t in params)
        if not (grad or on_dev):
            d, keep = sampler_desc(group, key, M, dev)
            pts, nrm, dlt, w = _launch_sample(d, F, M, dev)
            del keep
            return group.with_samples(pts, nrm, dlt, w)
        # the surface as a device vector read by the kernels (python numbers
        # become device fills: no host-to-device copy, no device read)
        as_t = lambda x: x.to(device=dev, dtype=torch.float32) if isinstance(x, torch.Tensor) else \
            torch.full((1,), float(x), device=dev)
        theta = torch.cat([as_t(surf.curvature).reshape(1), as_t(surf.conic).reshape(1),
                           as_t(surf.aspheric).reshape(-1)])
        d, keep = sampler_desc(group, key, M, dev, surface=theta.detach())
        if grad:
            pts, nrm, dlt, w = _SampleFunction.apply(theta, d, keep, F, M)
        else:
            pts, nrm, dlt, w = _launch_sample(d, F, M, dev)
        return group.with_samples(pts, nrm, dlt, w)
