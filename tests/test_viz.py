"""Plotting data (iactrace_gb300.viz): hexagon polygons reproduce the
reference's patch geometry, extents and histograms are consistent."""
from __future__ import annotations

import math

import numpy as np
import torch

from iactrace_gb300 import viz, workloads as W
from iactrace_gb300.sensors import SquareSensor


def test_hex_polygons_geometry():
    cam = W.hex_camera(960)
    poly = viz.hex_pixel_polygons(cam)
    P = cam.n_pixels
    assert poly.shape == (P, 6, 2)
    c = np.asarray(cam.hex_centers, dtype=np.float64)
    assert np.abs(poly.mean(1) - c).max() < 1e-9  # centred on the pixel centres
    r = np.linalg.norm(poly - c[:, None, :], axis=-1)
    assert np.abs(r - cam.hex_size).max() < 1e-9  # circumradius hex_size
    # neighbouring pixels share an edge: the nearest other centre is at
    # sqrt(3) * size, and its polygon has two vertices in common
    d = np.linalg.norm(c[1:] - c[0], axis=1)
    j = 1 + int(np.argmin(d))
    assert abs(d.min() - math.sqrt(3) * cam.hex_size) < 1e-4
    shared = (np.linalg.norm(poly[0][:, None, :] - poly[j][None, :, :], axis=-1) < 1e-6).sum()
    assert shared == 2


def test_square_extent_and_histogram():
    cam = SquareSensor([0, 0, 15.0], [0, 0, 0], 32, 30, (-0.672, 0.672, -0.63, 0.63))
    ext = viz.square_extent(cam)
    assert np.allclose(ext, (-0.672, 0.672, -0.63, 0.63))
    g = torch.Generator().manual_seed(0)
    pts = torch.rand((5000, 2), generator=g) * 1.2 - 0.6
    pts[:10] = 1e10  # misses
    vals = torch.rand(5000, generator=g)
    h = viz.hit_histogram(pts, vals, (32, 30), ext)
    assert h.shape == (30, 32)
    inside = (pts[:, 0].abs() < 0.672) & (pts[:, 1].abs() < 0.63)
    assert abs(float(h.sum()) - float(vals[inside].double().sum())) < 1e-9
    cv = viz.color_values(h)
    assert cv.max() == 1.0 and cv.min() >= 0.0
