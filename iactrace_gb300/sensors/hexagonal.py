"""Hexagonal-pixel sensors (sensors/hexagonal.py of the reference).

Grid detection and the axial lookup table are built on the host at
construction, in float32 with the reference's operation order
(sensors/hexagonal.py:61-101); binning runs inside the render kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from ._pack import pack_cached
from .. import _native as N

SQRT3 = 1.7320508075688772
SQRT3_2 = 0.8660254037844386
SQRT3_3 = 0.5773502691896257


def _rotate(x, y, angle):
    """sensors/hexagonal.py:16-20 (float32)."""
    a = np.float32(angle)
    c, s = np.cos(a), np.sin(a)
    return c * x - s * y, s * x + c * y


def _cartesian_to_axial(x, y, size):
    """sensors/hexagonal.py:23-25 (pointy-top)."""
    size = np.float32(size)
    return (np.float32(SQRT3_3) * x - y / np.float32(3)) / size, (np.float32(2) * y / np.float32(3)) / size


def _axial_to_cartesian(q, r, size):
    """sensors/hexagonal.py:28-29."""
    return np.float32(size * SQRT3) * (q + r / np.float32(2)), np.float32(size * 1.5) * r


def _axial_round(q, r):
    """sensors/hexagonal.py:32-39 (np.round is half-to-even, as jnp.round)."""
    s = -q - r
    qi, ri, si = np.round(q), np.round(r), np.round(s)
    dq, dr, ds = np.abs(qi - q), np.abs(ri - r), np.abs(si - s)
    qi = np.where((dq > dr) & (dq > ds), -ri - si, qi)
    ri = np.where((dr > dq) & (dr > ds), -qi - si, ri)
    return qi, ri


def _hex_neighbor_offsets(rings: int):
    """sensors/hexagonal.py:50-58."""
    off = [(q, r) for q in range(-rings, rings + 1) for r in range(-rings, rings + 1)
           if max(abs(q), abs(r), abs(-q - r)) <= rings]
    return np.array([o[0] for o in off], np.int32), np.array([o[1] for o in off], np.int32)


def _detect_hex_grid(centers: np.ndarray):
    """sensors/hexagonal.py:61-80: size, rotation and offset of the grid."""
    c = np.asarray(centers, dtype=np.float32)
    n = len(c)
    diff = c[:, None, :] - c[None, :, :]
    dist_sq = diff[..., 0] * diff[..., 0] + diff[..., 1] * diff[..., 1]
    np.fill_diagonal(dist_sq, np.inf)
    min_dist = np.sqrt(dist_sq.min())
    idx = int(np.argmin(dist_sq))
    vec = diff[idx // n, idx % n]
    angle = np.mod(np.arctan2(vec[1], vec[0]), np.float32(np.pi / 3))
    offset = c[int(np.argmin(c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]))]
    return np.float32(min_dist / np.float32(SQRT3)), np.float32(angle), offset


def _build_lookup_table(centers: np.ndarray, hex_size, rotation, offset):
    """sensors/hexagonal.py:83-101: table[q - q_min, r - r_min] = pixel id, -1 elsewhere."""
    c = np.asarray(centers, dtype=np.float32)
    x, y = c[:, 0] - offset[0], c[:, 1] - offset[1]
    xr, yr = _rotate(x, y, -float(rotation))
    q, r = _cartesian_to_axial(xr, yr, hex_size)
    qi, ri = np.round(q).astype(np.int32), np.round(r).astype(np.int32)
    q_min, r_min = int(qi.min()), int(ri.min())
    table = np.full((int(qi.max()) - q_min + 1, int(ri.max()) - r_min + 1), -1, dtype=np.int32)
    table[qi - q_min, ri - r_min] = np.arange(len(c), dtype=np.int32)
    return table, q_min, r_min


class HexagonalSensor:
    """sensors/hexagonal.py:104-194: hard binning into hexagonal pixels."""

    kind = N.SENSOR_HEX

    def __init__(self, position, rotation, hex_centers, edge_width: float = 0.0):
        self.position = torch.as_tensor(position, dtype=torch.float32).reshape(3)
        self.rotation = torch.as_tensor(rotation, dtype=torch.float32).reshape(3)
        hc = np.asarray(hex_centers.cpu() if isinstance(hex_centers, torch.Tensor) else hex_centers,
                        dtype=np.float32).reshape(-1, 2)
        self.hex_centers = torch.from_numpy(hc.copy())
        self.n_pixels = len(hc)
        self.edge_width = float(edge_width)
        size, rot, offset = _detect_hex_grid(hc)
        self.hex_size = float(size)
        self.hex_inradius = float(np.float32(size * np.float32(SQRT3_2)))
        self.grid_rotation = float(rot)
        self.grid_offset = (float(offset[0]), float(offset[1]))
        table, self.q_min, self.r_min = _build_lookup_table(hc, self.hex_size, self.grid_rotation, offset)
        self.lookup_table = torch.from_numpy(table)
        self._dev_table = {}

    def get_accumulator_shape(self):
        return (self.n_pixels,)

    def pack(self, device) -> tuple[N.IactSensor, list]:
        """The iact_sensor_t of this sensor on `device` (cached while its pose
        tensors and scalar settings are unchanged)."""
        return pack_cached(self, device, self._pack)

    def _pack(self, device) -> tuple[N.IactSensor, list]:
        key = str(device)
        if key not in self._dev_table:
            self._dev_table[key] = self.lookup_table.to(device=device, dtype=torch.int32).contiguous()
        tab = self._dev_table[key]
        s = N.IactSensor()
        s.type = self.kind
        s.n_pixels = self.n_pixels
        s.pos[:] = [float(v) for v in self.position.tolist()]
        s.rot[:] = [float(v) for v in self.rotation.tolist()]
        s.hex_size = np.float32(self.hex_size)
        s.inradius = np.float32(self.hex_inradius)
        a = np.float32(-self.grid_rotation)
        s.grid_cos, s.grid_sin = np.cos(a), np.sin(a)
        s.off_x, s.off_y = np.float32(self.grid_offset[0]), np.float32(self.grid_offset[1])
        s.hex_sx = np.float32(self.hex_size * SQRT3)
        s.hex_sy = np.float32(self.hex_size * 1.5)
        ew = getattr(self, "edge_width", 0.0)
        s.edge_width = np.float32(ew)
        s.edge_threshold = np.float32(1.0 - ew / self.hex_inradius)
        s.q_min, s.r_min = self.q_min, self.r_min
        s.table_q, s.table_r = int(tab.shape[0]), int(tab.shape[1])
        s.table = tab.data_ptr()
        s.sigma = np.float32(getattr(self, "sigma", 0.0))
        s.kernel_size = int(getattr(self, "kernel_size", 0))
        return s, [tab]


class DifferentiableHexagonalSensor(HexagonalSensor):
    """sensors/hexagonal.py:197-315: Gaussian splat on the hex norm over
    `kernel_size` neighbour rings, sigma in units of the inradius."""

    kind = N.SENSOR_SOFT_HEX

    def __init__(self, position, rotation, hex_centers, sigma: float = 0.5, kernel_size: int = 1):
        super().__init__(position, rotation, hex_centers, 0.0)
        self.sigma = float(sigma)
        self.kernel_size = int(kernel_size)
