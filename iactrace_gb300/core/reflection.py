"""Reflection and roughness deltas (core/reflection.py of the reference)."""
from __future__ import annotations

import torch


def reflect(d, n):
    """core/reflection.py:5-20: r = d - 2 (d.n) n, returns (r, -(d.n))."""
    c = torch.sum(d * n, dim=-1, keepdim=True)
    return d - 2.0 * c * n, -c


def perturbation_delta_from_normals(normals, theta1, theta2):
    """core/reflection.py:22-49 with the two N(0,1) draws given: tangent basis
    from cross(n, ref) with ref = x if |n_z| > 0.9 else z."""
    ref_z = torch.tensor([0.0, 0.0, 1.0], dtype=normals.dtype, device=normals.device)
    ref_x = torch.tensor([1.0, 0.0, 0.0], dtype=normals.dtype, device=normals.device)
    dot_z = torch.abs(torch.sum(normals * ref_z, dim=-1, keepdim=True))
    ref = torch.where(dot_z > 0.9, ref_x, ref_z)
    t1 = torch.linalg.cross(normals, ref.expand_as(normals))
    t1 = t1 / torch.linalg.norm(t1, dim=-1, keepdim=True)
    t2 = torch.linalg.cross(normals, t1)
    return theta1[..., None] * t1 + theta2[..., None] * t2


def compute_perturbation_delta(normals, gen: torch.Generator | None = None):
    """core/reflection.py:22-49: unit-sigma tangent-space deltas."""
    shape = normals.shape[:-1]
    th1 = torch.randn(shape, generator=gen, dtype=normals.dtype)
    th2 = torch.randn(shape, generator=gen, dtype=normals.dtype)
    return perturbation_delta_from_normals(normals, th1, th2)
