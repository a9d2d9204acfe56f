"""Mirrors and mirror groups (telescope/mirrors.py of the reference).

Groups are SoA containers of torch tensors. Stage-0 groups carry the sampled
geometry the render path traces from; stage >= 1 groups are intersected by
the render kernels (core/render.py:44-115).
"""
from __future__ import annotations

import copy
from collections import defaultdict

import torch

from ..core.apertures import DiskAperture, PolygonAperture
from ..core.surfaces import AsphericSurface
from ..core.transforms import euler_to_matrix


def _t(x):
    return torch.as_tensor(x, dtype=torch.float32)


class Mirror:
    """telescope/mirrors.py:10-43: one mirror element."""

    def __init__(self, position, rotation, surface, aperture, points=None, normals=None, weights=None,
                 optical_stage=0, offset=None):
        self.position = _t(position).reshape(3)
        self.rotation = _t(rotation).reshape(3)
        self.surface = surface
        self.aperture = aperture
        self.offset = _t(offset).reshape(2) if offset is not None else torch.zeros(2)
        self.points = points if points is not None else torch.zeros((0, 3))
        self.normals = normals if normals is not None else torch.zeros((0, 3))
        self.weights = weights if weights is not None else torch.zeros((0, 1))
        self.optical_stage = int(optical_stage)

    def transform_to_world(self):
        """telescope/mirrors.py:38-43."""
        R = euler_to_matrix(self.rotation)
        return self.points @ R.T + self.position, self.normals @ R.T, self.weights


class MirrorGroup:
    """telescope/mirrors.py:46-98: per-mirror transforms + per-sample geometry.

    positions (N,3), rotations (N,3) Euler degrees, points/normals/
    perturbation_delta (N,M,3) local, weights (N,M,1), perturbation_scale (N,)
    radians, optical_stage.
    """

    def _init_common(self, positions, rotations, surface, optical_stage, offsets):
        self.positions = _t(positions).reshape(-1, 3)
        self.rotations = _t(rotations).reshape(-1, 3)
        # floats, or 0-d tensors when they are optimised (stage >= 1 mirrors)
        self.curvature = surface.curvature if isinstance(surface.curvature, torch.Tensor) else float(surface.curvature)
        self.conic = surface.conic if isinstance(surface.conic, torch.Tensor) else float(surface.conic)
        self.aspheric = surface.aspheric.clone()
        self.optical_stage = int(optical_stage)
        n = self.positions.shape[0]
        self.offsets = _t(offsets).reshape(-1, 2) if offsets is not None else torch.zeros((n, 2))
        self.points = torch.zeros((n, 0, 3))
        self.normals = torch.zeros((n, 0, 3))
        self.weights = torch.zeros((n, 0, 1))
        self.perturbation_delta = torch.zeros((n, 0, 3))
        self.perturbation_scale = torch.zeros(n)

    def __len__(self):
        return self.positions.shape[0]

    @property
    def n_samples(self) -> int:
        return int(self.points.shape[1])

    def get_surface(self) -> AsphericSurface:
        return AsphericSurface(self.curvature, self.conic, self.aspheric)

    def replace(self, **fields) -> "MirrorGroup":
        """Functional update (the reference's eqx.tree_at)."""
        g = copy.copy(self)
        for k, v in fields.items():
            setattr(g, k, v)
        return g

    def with_samples(self, points, normals, delta, weights) -> "MirrorGroup":
        return self.replace(points=points, normals=normals, perturbation_delta=delta, weights=weights)

    def transform_to_world(self):
        """telescope/mirrors.py:64-79 (host version; the kernels do this on device)."""
        R = euler_to_matrix(self.rotations)  # (N,3,3)
        pw = torch.einsum("nij,nmj->nmi", R, self.points) + self.positions[:, None, :]
        nw = torch.einsum("nij,nmj->nmi", R, self.normals)
        dw = torch.einsum("nij,nmj->nmi", R, self.perturbation_delta)
        pe = nw + self.perturbation_scale[:, None, None] * dw
        return pw, pe / torch.linalg.norm(pe, dim=-1, keepdim=True), self.weights

    def check_aperture(self, x, y, mirror_idx):
        raise NotImplementedError

    def get_sampling_params(self):
        raise NotImplementedError


class AsphericDiskMirrorGroup(MirrorGroup):
    """telescope/mirrors.py:101-158: shared surface, per-mirror disk radius."""

    def __init__(self, positions, rotations, surface, radii, optical_stage=0, offsets=None):
        self._init_common(positions, rotations, surface, optical_stage, offsets)
        self.radii = _t(radii).reshape(-1)

    def check_aperture(self, x, y, mirror_idx):
        return x ** 2 + y ** 2 <= self.radii[mirror_idx] ** 2

    def get_sampling_params(self):
        return {"type": "disk", "radii": self.radii, "offsets": self.offsets, "surface": self.get_surface()}


class AsphericPolygonMirrorGroup(MirrorGroup):
    """telescope/mirrors.py:161-229: shared surface, per-mirror convex polygon."""

    def __init__(self, positions, rotations, surface, vertices_list, optical_stage=0, offsets=None):
        self._init_common(positions, rotations, surface, optical_stage, offsets)
        self.vertices = _t(vertices_list)
        self.n_vertices = int(self.vertices.shape[1])

    def check_aperture(self, x, y, mirror_idx):
        v = self.vertices[mirror_idx]
        n = self.n_vertices
        inside = torch.ones_like(torch.as_tensor(x), dtype=torch.bool)
        for i in range(n):
            a, b = v[i], v[(i + 1) % n]
            inside = inside & ((b[0] - a[0]) * (y - a[1]) - (b[1] - a[1]) * (x - a[0]) >= 0)
        return inside

    def get_sampling_params(self):
        return {"type": "polygon", "vertices": self.vertices, "offsets": self.offsets,
                "surface": self.get_surface()}


def _group_by_surface_params(mirrors):
    """telescope/mirrors.py:316-335."""
    grouped = defaultdict(list)
    for m in mirrors:
        if isinstance(m.surface, AsphericSurface):
            grouped[m.surface.key()].append(m)
    return grouped


def group_mirrors(mirrors):
    """telescope/mirrors.py:232-313: by stage, then disk groups by surface,
    then polygon groups by vertex count and surface."""
    if not mirrors:
        return []
    by_stage = defaultdict(list)
    for m in mirrors:
        by_stage[m.optical_stage].append(m)
    groups = []
    for stage, sm in sorted(by_stage.items()):
        disk = [m for m in sm if isinstance(m.surface, AsphericSurface) and isinstance(m.aperture, DiskAperture)]
        for _, ml in _group_by_surface_params(disk).items():
            groups.append(AsphericDiskMirrorGroup(
                torch.stack([m.position for m in ml]), torch.stack([m.rotation for m in ml]), ml[0].surface,
                [m.aperture.radius for m in ml], optical_stage=stage, offsets=torch.stack([m.offset for m in ml])))
        poly = [m for m in sm if isinstance(m.surface, AsphericSurface) and isinstance(m.aperture, PolygonAperture)]
        by_nv = defaultdict(list)
        for m in poly:
            by_nv[m.aperture.n_vertices].append(m)
        for _, mlist in by_nv.items():
            for _, ml in _group_by_surface_params(mlist).items():
                groups.append(AsphericPolygonMirrorGroup(
                    torch.stack([m.position for m in ml]), torch.stack([m.rotation for m in ml]), ml[0].surface,
                    torch.stack([m.aperture.vertices for m in ml]), optical_stage=stage,
                    offsets=torch.stack([m.offset for m in ml])))
    return groups
