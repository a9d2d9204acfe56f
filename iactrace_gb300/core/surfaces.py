"""Aspheric surface (core/surfaces.py of the reference).

Host-side (torch) evaluation used by scene construction and the sampler's
reference mapping; the render kernels carry their own device copy of the
same sag / normal / ray-intersection math.
"""
from __future__ import annotations

import torch


class AsphericSurface:
    """core/surfaces.py:8: curvature c, conic k and coefficients a_i of r^(4(i+1))."""

    def __init__(self, curvature, conic, aspheric=()):
        # floats, or 0-d tensors when they are optimised
        self.curvature = curvature if isinstance(curvature, torch.Tensor) else float(curvature)
        self.conic = conic if isinstance(conic, torch.Tensor) else float(conic)
        self.aspheric = aspheric if isinstance(aspheric, torch.Tensor) else \
            torch.as_tensor(aspheric, dtype=torch.float32)
        self.aspheric = self.aspheric.reshape(-1)

    @staticmethod
    def from_template(tmpl) -> "AsphericSurface":
        """core/surfaces.py:15-23."""
        s = tmpl["surface"]
        return AsphericSurface(float(s["curvature"]), float(s["conic"]), s.get("aspheric", []) or [])

    def key(self):
        v = lambda x: float(x.detach()) if isinstance(x, torch.Tensor) else float(x)
        return (v(self.curvature), v(self.conic), tuple(float(a) for a in self.aspheric.detach().tolist()))

    def _sag_raw(self, x, y):
        """core/surfaces.py:25-39 (aspheric term i multiplies r2**(2(i+1)))."""
        r2 = x * x + y * y
        c, k = self.curvature, self.conic
        z = r2 * c / (1 + torch.sqrt(1 - (1 + k) * c * c * r2))
        a = self.aspheric.to(device=r2.device, dtype=r2.dtype)
        for i in range(a.shape[0]):  # tensor ops: the coefficients may carry gradients
            z = z + a[i] * r2 ** (2 * (i + 1))
        return z

    def _sag_raw_dr2(self, r2):
        c, k = self.curvature, self.conic
        alpha = (1 + k) * c * c
        s = torch.sqrt(1 - alpha * r2)
        den = 1 + s
        dz = c / den + (r2 * c) * alpha / (2 * s * den * den)
        a = self.aspheric.to(device=r2.device, dtype=r2.dtype)
        for i in range(a.shape[0]):
            p = 2 * (i + 1)
            dz = dz + a[i] * p * r2 ** (p - 1)
        return dz

    def sag(self, x, y, offset):
        """core/surfaces.py:41-45."""
        x0, y0 = offset[..., 0], offset[..., 1]
        return self._sag_raw(x + x0, y + y0) - self._sag_raw(x0, y0)

    def point(self, x, y, offset):
        """core/surfaces.py:47-49."""
        return torch.stack([x, y, self.sag(x, y, offset)], dim=-1)

    def normal(self, x, y, offset):
        """core/surfaces.py:51-58 (analytic gradient of the sag)."""
        xs, ys = x + offset[..., 0], y + offset[..., 1]
        g = self._sag_raw_dr2(xs * xs + ys * ys)
        n = torch.stack([-(g * 2 * xs), -(g * 2 * ys), torch.ones_like(xs)], dim=-1)
        return n / torch.linalg.norm(n, dim=-1, keepdim=True)

    def point_and_normal(self, xy, offset):
        """core/surfaces.py:60-65."""
        x, y = xy[..., 0], xy[..., 1]
        return self.point(x, y, offset), self.normal(x, y, offset)
