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
from .reflection import compute_perturbation_delta, perturbation_delta_from_normals


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


def sampler_desc(group, key, n_samples: int, device):
    """The iact_sampler_t of a stage-0 group and its arrays on `device`
    (returns the descriptor and the tensors it points at)."""
    params = group.get_sampling_params()
    surf = params["surface"]
    d = N.IactSampler()
    d.n_facets, d.n_samples = len(group), int(n_samples)
    value = lambda x: float(x.detach()) if isinstance(x, torch.Tensor) else float(x)
    d.curvature, d.conic = value(surf.curvature), value(surf.conic)
    a = surf.aspheric.detach().reshape(-1).tolist()
    if len(a) > N.IACT_MAX_ASPH:
        raise ValueError(f"at most {N.IACT_MAX_ASPH} aspheric coefficients")
    d.n_asph = len(a)
    for i, v in enumerate(a):
        d.asph[i] = float(v)
    keep = [params["offsets"].reshape(-1, 2).to(device=device, dtype=torch.float32).contiguous()]
    d.offsets = keep[0].data_ptr()
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


class DeviceIntegrator(Integrator):
    """MCIntegrator on the GPU: same aperture, surface, roughness-delta and
    weight construction (core/integrators.py:97-187), variates from the
    counter-based stream of iact_sample_facets (reproducible on any host)."""

    def __init__(self, n_samples: int = 128, device=None):
        self.n_samples = int(n_samples)
        self.device = device

    def sample_group(self, group, key):
        dev = torch.device(self.device) if self.device is not None else torch.device("cuda", torch.cuda.current_device())
        d, keep = sampler_desc(group, key, self.n_samples, dev)
        F, M = len(group), self.n_samples
        pts, nrm, dlt = (torch.empty((F, M, 3), device=dev) for _ in range(3))
        w = torch.empty((F, M, 1), device=dev)
        lib = N.load()
        N.check(lib.iact_sample_facets(ctypes.byref(d), pts.data_ptr(), nrm.data_ptr(), dlt.data_ptr(), w.data_ptr(),
                                       torch.cuda.current_stream(dev).cuda_stream))
        del keep
        surf = group.get_surface()
        params = [surf.curvature, surf.conic, surf.aspheric]
        if any(isinstance(t, torch.Tensor) and t.requires_grad for t in params):
            pts, nrm, dlt, w = self._differentiable(group, surf, pts, nrm, dlt, w)
        return group.with_samples(pts, nrm, dlt, w)

    def _differentiable(self, group, surf, pts, nrm, dlt, w):
        """The sample arrays as functions of the surface parameters (FP64
        torch restatement of the kernel's mapping, core/surfaces.py:41-65 and
        core/reflection.py:22-49): the aperture positions and the roughness
        coefficients do not depend on the surface; points, normals, deltas
        and weights do (resampling gradients)."""
        dev = pts.device
        xy = pts[..., :2].double()
        n0 = nrm.double()
        # the roughness coefficients of the drawn deltas in their tangent basis
        ref_z = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64, device=dev)
        ref_x = torch.tensor([1.0, 0.0, 0.0], dtype=torch.float64, device=dev)
        ref = torch.where(n0[..., 2:3].abs() > 0.9, ref_x, ref_z)
        t1 = torch.linalg.cross(n0, ref.expand_as(n0))
        t1 = t1 / torch.linalg.norm(t1, dim=-1, keepdim=True)
        t2 = torch.linalg.cross(n0, t1)
        d0 = dlt.double()
        th1, th2 = (d0 * t1).sum(-1), (d0 * t2).sum(-1)
        s64 = type(surf)(surf.curvature if not isinstance(surf.curvature, torch.Tensor) else surf.curvature.double(),
                         surf.conic if not isinstance(surf.conic, torch.Tensor) else surf.conic.double(),
                         surf.aspheric.double())
        off = group.offsets.reshape(-1, 1, 2).to(device=dev, dtype=torch.float64)
        p, n = s64.point_and_normal(xy, off)
        dl = perturbation_delta_from_normals(n, th1, th2)
        area = (n0[..., 2] / w[..., 0].double() * self.n_samples).detach()  # per facet: pi R^2 or polygon area
        ww = n[..., 2:3] / area[..., None] * self.n_samples
        return p.float(), n.float(), dl.float(), ww.float()
