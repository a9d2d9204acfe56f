"""Monte-Carlo facet sampling (core/integrators.py of the reference).

``MCIntegrator.sample_group`` fills a stage-0 mirror group with local sample
points, unit normals, unit-sigma roughness deltas and weights
``cos_z / area * n_samples`` (core/integrators.py:97-187).
"""
from __future__ import annotations

import math
from abc import ABC, abstractmethod

import torch

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
