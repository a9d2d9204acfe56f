"""Mirror apertures (core/apertures.py of the reference)."""
from __future__ import annotations

import math

import torch


class Aperture:
    def area(self):
        raise NotImplementedError

    def check_aperture(self, x, y):
        raise NotImplementedError


class DiskAperture(Aperture):
    """core/apertures.py:22-34."""

    def __init__(self, radius: float = 1.0):
        self.radius = float(radius)

    def area(self):
        return math.pi * self.radius ** 2

    def check_aperture(self, x, y):
        return x ** 2 + y ** 2 <= self.radius ** 2


class PolygonAperture(Aperture):
    """core/apertures.py:37-63: convex polygon, inside = every edge cross >= 0."""

    def __init__(self, vertices):
        self.vertices = torch.as_tensor(vertices, dtype=torch.float32).reshape(-1, 2)
        self.n_vertices = int(self.vertices.shape[0])

    def area(self):
        x, y = self.vertices[:, 0], self.vertices[:, 1]
        return 0.5 * torch.abs(torch.sum(x * torch.roll(y, -1) - torch.roll(x, -1) * y))

    def check_aperture(self, x, y):
        inside = torch.ones_like(torch.as_tensor(x), dtype=torch.bool)
        v = self.vertices
        n = self.n_vertices
        for i in range(n):
            a, b = v[i], v[(i + 1) % n]
            cross = (b[0] - a[0]) * (y - a[1]) - (b[1] - a[1]) * (x - a[0])
            inside = inside & (cross >= 0)
        return inside
