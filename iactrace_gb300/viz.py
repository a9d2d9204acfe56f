"""Plotting data (viz/plotting.py of the reference, data only).

The reference draws square images with ``imshow`` and hexagonal images as
one matplotlib ``RegularPolygon`` per pixel (viz/plotting.py:6-82). This
module returns what those plots need, as arrays, and draws nothing: the
extent of a square image, the vertices of every hexagonal pixel (the
reference's patch geometry: pointy-top hexagons of circumradius hex_size,
turned by minus the grid rotation), colour values normalised as the
reference normalises them, and a 2-D histogram of raw hits from
``render_debug`` (spot and point-spread-function maps).
"""
from __future__ import annotations

import math

import numpy as np
import torch


def square_extent(sensor):
    """viz/plotting.py:6-34 squareshow: imshow extent (x0, x1, y0, y1) of a
    square sensor's (H, W) image, origin lower."""
    return (float(sensor.x0), float(sensor.x0 + sensor.width * sensor.dx),
            float(sensor.y0), float(sensor.y0 + sensor.height * sensor.dy))


def hex_pixel_polygons(sensor) -> np.ndarray:
    """viz/plotting.py:37-82 hexshow: the 6 vertices (P, 6, 2) of every
    pixel, as RegularPolygon(centre, 6, radius=hex_size,
    orientation=-grid_rotation) places them (first vertex straight up for
    orientation 0, then counter-clockwise)."""
    c = np.asarray(sensor.hex_centers, dtype=np.float64)
    ang = math.pi / 2 - float(sensor.grid_rotation) + 2 * math.pi * np.arange(6) / 6
    off = float(sensor.hex_size) * np.stack([np.cos(ang), np.sin(ang)], -1)  # (6, 2)
    return c[:, None, :] + off[None, :, :]


def color_values(result, vmin=None, vmax=None) -> np.ndarray:
    """The colour-map argument hexshow passes per pixel:
    clip(value, vmin, inf) / vmax, vmin and vmax defaulting to the data's
    min and max (viz/plotting.py:60-72)."""
    r = np.asarray(result.detach().cpu() if isinstance(result, torch.Tensor) else result, dtype=np.float64)
    lo = r.min() if vmin is None else vmin
    hi = r.max() if vmax is None else vmax
    return np.clip(r, lo, np.inf) / hi


def hit_histogram(pts, vals, bins, extent) -> torch.Tensor:
    """Value-weighted 2-D histogram (ny, nx) of raw sensor-plane hits
    (render_debug's pts (N, 2), vals (N,)) over extent (x0, x1, y0, y1);
    the 1e10 miss sentinel and hits outside the extent are dropped. Runs
    where the hits are (device tensors stay on the device)."""
    nx, ny = (bins, bins) if isinstance(bins, int) else bins
    x0, x1, y0, y1 = extent
    x, y = pts[:, 0], pts[:, 1]
    ix = torch.floor((x - x0) / (x1 - x0) * nx).long()
    iy = torch.floor((y - y0) / (y1 - y0) * ny).long()
    ok = (ix >= 0) & (ix < nx) & (iy >= 0) & (iy < ny) & (x < 1e9) & (y < 1e9)
    out = torch.zeros(ny * nx, dtype=torch.float64, device=pts.device)
    out.index_add_(0, (iy * nx + ix)[ok], vals[ok].double())
    return out.reshape(ny, nx)
