"""Euler-angle rotations (core/transforms.py of the reference).

``euler_to_matrix`` restates core/transforms.py:72-107: degrees (tip, tilt,
rotation) -> R = Rz @ Ry @ Rx. The render kernels evaluate the same matrix
on the device; these host versions serve scene construction and tooling.
"""
from __future__ import annotations

import math

import torch


def _as_tensor(x, dtype=torch.float32):
    return x if isinstance(x, torch.Tensor) else torch.as_tensor(x, dtype=dtype)


def euler_to_matrix(tip_tilt_rotation) -> torch.Tensor:
    """core/transforms.py:72-107; batched over leading dimensions."""
    a = _as_tensor(tip_tilt_rotation)
    r = torch.deg2rad(a)
    cx, cy, cz = torch.cos(r[..., 0]), torch.cos(r[..., 1]), torch.cos(r[..., 2])
    sx, sy, sz = torch.sin(r[..., 0]), torch.sin(r[..., 1]), torch.sin(r[..., 2])
    # Rz @ Ry @ Rx written out (elementwise: no batched GEMM)
    return torch.stack([cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx,
                        sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx,
                        -sy, cy * sx, cy * cx], -1).reshape(*cx.shape, 3, 3)


def look_at_rotation(mirror_pos, target_pos=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> torch.Tensor:
    """core/transforms.py:4-24: columns (right, up, forward) looking at target."""
    p, t, u = (_as_tensor(v, torch.float64) for v in (mirror_pos, target_pos, up))
    fwd = t - p
    fwd = fwd / torch.linalg.norm(fwd)
    right = torch.linalg.cross(fwd, u)
    right = right / torch.linalg.norm(right)
    upc = torch.linalg.cross(right, fwd)
    return torch.stack([right, upc, fwd], dim=1)


def look_at_euler(mirror_pos, target_pos=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> torch.Tensor:
    """core/transforms.py:27-69: Euler degrees (tip, tilt, rotation) of a look-at frame."""
    p, t, u = (_as_tensor(v, torch.float64) for v in (mirror_pos, target_pos, up))
    fwd = t - p
    fwd = fwd / torch.linalg.norm(fwd)
    right = torch.linalg.cross(u, fwd)
    right = right / torch.linalg.norm(right)
    upc = torch.linalg.cross(fwd, right)
    R = torch.stack([right, upc, fwd], dim=1)
    sy = -R[2, 0]
    cy = math.sqrt(max(0.0, 1.0 - float(sy) ** 2))
    if cy > 1e-6:
        tip = math.atan2(float(R[2, 1]), float(R[2, 2]))
        rot = math.atan2(float(R[1, 0]), float(R[0, 0]))
    else:
        tip = 0.0
        rot = math.atan2(float(-R[0, 1]), float(R[1, 1]))
    tilt = math.asin(float(sy))
    return torch.tensor([math.degrees(tip), math.degrees(tilt), math.degrees(rot)], dtype=torch.float32)
