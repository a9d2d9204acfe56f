"""Square-pixel sensors (sensors/square.py of the reference).

Construction computes the float32 constants the reference derives at
construction time; binning itself runs inside the render kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from ._pack import pack_cached
from .. import _native as N


def _t(x):
    return torch.as_tensor(x, dtype=torch.float32)


class SquareSensor:
    """sensors/square.py:28-91: hard binning with an optional edge band."""

    kind = N.SENSOR_SQUARE

    def __init__(self, position, rotation, width: int, height: int, bounds, edge_width: float = 0.0):
        self.position = _t(position).reshape(3)
        self.rotation = _t(rotation).reshape(3)
        self.width, self.height = int(width), int(height)
        self.edge_width = float(edge_width)
        xmin, xmax, ymin, ymax = (float(b) for b in bounds)
        self.x0, self.y0 = xmin, ymin
        self.dx = (xmax - xmin) / self.width
        self.dy = (ymax - ymin) / self.height

    def get_accumulator_shape(self):
        return (self.height, self.width)

    @property
    def n_pixels(self) -> int:
        return self.width * self.height

    def pack(self, device) -> tuple[N.IactSensor, list]:
        """The iact_sensor_t of this sensor on `device` (cached while its pose
        tensors and scalar settings are unchanged)."""
        return pack_cached(self, device, self._pack)

    def _pack(self, device) -> tuple[N.IactSensor, list]:
        s = N.IactSensor()
        s.type = self.kind
        s.n_pixels = self.n_pixels
        s.width, s.height = self.width, self.height
        s.pos[:] = [float(v) for v in self.position.tolist()]
        s.rot[:] = [float(v) for v in self.rotation.tolist()]
        s.x0, s.y0 = np.float32(self.x0), np.float32(self.y0)
        s.dx, s.dy = np.float32(self.dx), np.float32(self.dy)
        s.edge_width = np.float32(getattr(self, "edge_width", 0.0))
        s.sigma = np.float32(getattr(self, "sigma", 0.0))
        s.kernel_size = int(getattr(self, "kernel_size", 0))
        return s, []


class DifferentiableSquareSensor(SquareSensor):
    """sensors/square.py:94-172: Gaussian soft splat over (2K+1)^2 pixels,
    sigma in pixel units, weights normalised per ray."""

    kind = N.SENSOR_SOFT_SQUARE

    def __init__(self, position, rotation, width: int, height: int, bounds=(-1, 1, -1, 1), sigma: float = 0.1,
                 kernel_size: int = 2):
        super().__init__(position, rotation, width, height, bounds, 0.0)
        self.sigma = float(sigma)
        self.kernel_size = int(kernel_size)
