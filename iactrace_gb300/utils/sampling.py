"""Samplers of the Monte-Carlo integrator (utils/sampling.py of the reference).

The functions map uniform variates to points; ``u`` arguments let a caller
(or a test) feed the variates explicitly, otherwise they are drawn from the
given torch.Generator.
"""
from __future__ import annotations

import math

import torch


def sample_disk(gen: torch.Generator | None, shape, u1=None, u2=None, dtype=torch.float32):
    """utils/sampling.py:8-27: r = sqrt(u1), theta = 2 pi u2, unit disk."""
    if u1 is None:
        u1 = torch.rand(shape, generator=gen, dtype=dtype)
    if u2 is None:
        u2 = torch.rand(shape, generator=gen, dtype=dtype)
    r = torch.sqrt(u1)
    th = u2 * 2 * math.pi
    return torch.stack([r * torch.cos(th), r * torch.sin(th)], dim=-1)


def polygon_triangles(vertices: torch.Tensor):
    """Fan triangulation from vertex 0 and its area-proportional weights."""
    n = vertices.shape[-2]
    tri = torch.stack([torch.stack([vertices[..., 0, :], vertices[..., i, :], vertices[..., i + 1, :]], -2)
                       for i in range(1, n - 1)], -3)  # (..., n-2, 3, 2)
    v0, v1, v2 = tri[..., 0, :], tri[..., 1, :], tri[..., 2, :]
    areas = torch.abs((v1[..., 0] - v0[..., 0]) * (v2[..., 1] - v0[..., 1])
                      - (v2[..., 0] - v0[..., 0]) * (v1[..., 1] - v0[..., 1])) / 2
    return tri, areas / areas.sum(-1, keepdim=True)


def sample_polygon(gen: torch.Generator | None, vertices, shape, uc=None, u1=None, u2=None,
                   dtype=torch.float32):
    """utils/sampling.py:30-67: area-weighted fan triangle, then a uniform
    point in it via (1 - sqrt(u), sqrt(u)(1 - v), sqrt(u) v)."""
    vertices = torch.as_tensor(vertices, dtype=dtype)
    tri, probs = polygon_triangles(vertices)
    if uc is None:
        uc = torch.rand(shape, generator=gen, dtype=dtype)
    cdf = torch.cumsum(probs, 0)
    idx = torch.clamp(torch.searchsorted(cdf, uc.contiguous(), right=True), max=tri.shape[0] - 1)
    if u1 is None:
        u1 = torch.rand(shape, generator=gen, dtype=dtype)
    if u2 is None:
        u2 = torch.rand(shape, generator=gen, dtype=dtype)
    u = torch.sqrt(u1)
    a, b, c = 1 - u, u * (1 - u2), u * u2
    tv = tri[idx]
    return a[..., None] * tv[..., 0, :] + b[..., None] * tv[..., 1, :] + c[..., None] * tv[..., 2, :]
