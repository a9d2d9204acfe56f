"""Synthetic telescope scenes of the benchmark workloads (seeded, no files).

  davies_cotton()        12 m Davies-Cotton dish, f = 15 m, 380 spherical hex
                         facets (0.60 m flat-to-flat, R = 2f), Gaussian
                         tip/tilt errors (sigma 0.5 mrad), 4 mast cylinders
                         (r = 5 cm) and a 1.5 x 1.5 x 1.6 m camera box.
  plain_forward()        that dish, 32 x 30 square camera (42 mm pitch),
                         16 point sources at z = 1e10 within 2.5 deg, values
                         U(0.5, 1), 1000 samples per facet.
  response_matrix()      that dish, 2048-pixel hex camera (42 mm pitch),
                         4096 point sources on a 64 x 64 grid within +-3 deg,
                         unit values, 256 samples per facet.
  cassegrain()           two-mirror Cassegrain: 10 m conic primary
                         (k = -1.05, f = 10 m) of 61 hex segments with
                         aspheric terms, 3 m hyperboloid secondary, 32 x 32
                         square camera, 64 point sources within 1.5 deg.
  ragged_batch()         64 Davies-Cotton variants: the first n (uniform
                         100..900) facets of one 900-facet dish, tip/tilt
                         errors with sigma uniform in 0.2..1.0 mrad, 960- or
                         2048-pixel hex camera, log-uniform 1..4096 point
                         sources within 2.5 deg, 256 samples per facet.

Facet layouts follow the Davies-Cotton construction: facet centres on a
sphere of radius f about the focus, each facet normal aimed at (0, 0, 2f).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .core.apertures import DiskAperture, PolygonAperture
from .core.integrators import MCIntegrator
from .core.obstructions import Box, Cylinder, group_obstructions
from .core.surfaces import AsphericSurface
from .sensors import HexagonalSensor, SquareSensor
from .telescope.mirrors import Mirror, group_mirrors
from .telescope.telescope import Telescope
from .utils import keys as _keys


def hex_grid(n: int, pitch: float) -> np.ndarray:
    """The n points of a pointy-top hexagonal lattice (nearest-neighbour
    distance `pitch`) closest to the origin, ordered by radius then angle."""
    rings = int(math.ceil(math.sqrt(n / 3.0))) + 3
    pts = []
    for q in range(-rings, rings + 1):
        for r in range(-rings, rings + 1):
            x = pitch * (q + r / 2.0)
            y = pitch * (math.sqrt(3) / 2.0) * r
            pts.append((x, y))
    pts = np.array(pts)
    rad = np.round(np.hypot(pts[:, 0], pts[:, 1]), 9)
    ang = np.round(np.mod(np.arctan2(pts[:, 1], pts[:, 0]), 2 * np.pi), 9)
    order = np.lexsort((ang, rad))
    return pts[order[:n]]


def hex_vertices(flat_to_flat: float) -> list[list[float]]:
    """Counter-clockwise vertices of a pointy-top hexagon."""
    rc = flat_to_flat / math.sqrt(3.0)
    return [[rc * math.cos(math.radians(90 + 60 * k)), rc * math.sin(math.radians(90 + 60 * k))] for k in range(6)]


def dc_orientation(pos, aim_z: float) -> list[float]:
    """Euler (tip, tilt, 0) degrees whose local +z points from pos to (0, 0, aim_z)."""
    nvec = np.array([-pos[0], -pos[1], aim_z - pos[2]], float)
    nvec /= np.linalg.norm(nvec)
    tip = -math.degrees(math.asin(nvec[1]))
    tilt = math.degrees(math.atan2(nvec[0], nvec[2]))
    return [tip, tilt, 0.0]


def davies_cotton(n_facets: int = 380, focal: float = 15.0, facet_flat: float = 0.60, tilt_sigma_mrad: float = 0.5,
                  n_samples: int = 1000, seed: int = 0, obstructions: bool = True):
    """Mirror groups (sampled) and obstruction groups of the DC dish."""
    rng = np.random.default_rng(seed)
    centres = hex_grid(n_facets, facet_flat)
    surf = AsphericSurface(curvature=1.0 / (2.0 * focal), conic=0.0, aspheric=[])
    verts = hex_vertices(facet_flat)
    sig_deg = math.degrees(tilt_sigma_mrad * 1e-3)
    mirrors = []
    for (x, y) in centres:
        z = focal - math.sqrt(focal * focal - x * x - y * y)
        rot = dc_orientation((x, y, z), 2.0 * focal)
        rot[0] += sig_deg * rng.standard_normal()
        rot[1] += sig_deg * rng.standard_normal()
        mirrors.append(Mirror([x, y, z], rot, surf, PolygonAperture(verts), optical_stage=0))
    groups = group_mirrors(mirrors)
    key = _keys.key(seed)
    integ = MCIntegrator(n_samples)
    groups = [integ.sample_group(g, k) for g, k in zip(groups, _keys.split(key, len(groups)))]
    obst = []
    if obstructions:
        rim = 0.5 * facet_flat * math.sqrt(n_facets * math.sqrt(3) / 2 / math.pi) * 2 * 1.15
        for ang in (60.0, 120.0, 240.0, 300.0):
            a = math.radians(ang)
            p1 = [rim * math.cos(a), rim * math.sin(a), 1.2]
            p2 = [1.155 * math.cos(a), 1.155 * math.sin(a), focal + 0.6]
            obst.append(Cylinder(p1, p2, 0.05))
        obst.append(Box([-0.75, -0.75, focal], [0.75, 0.75, focal + 1.6]))
    return groups, group_obstructions(obst)


def point_sources_disk(n: int, max_deg: float, seed: int, distance: float = 1e10):
    """n point sources at z = distance, directions uniform in a disk of angular radius max_deg."""
    g = torch.Generator().manual_seed(seed)
    th = torch.deg2rad(torch.tensor(max_deg, dtype=torch.float64)) * torch.sqrt(torch.rand(n, generator=g, dtype=torch.float64))
    ph = 2 * math.pi * torch.rand(n, generator=g, dtype=torch.float64)
    t = torch.tan(th)
    return torch.stack([distance * t * torch.cos(ph), distance * t * torch.sin(ph),
                        torch.full((n,), distance, dtype=torch.float64)], 1).float()


def point_sources_grid(n_side: int, half_deg: float, distance: float = 1e10):
    """n_side^2 point sources at z = distance on a regular angle grid within +-half_deg."""
    a = torch.deg2rad(torch.linspace(-half_deg, half_deg, n_side, dtype=torch.float64))
    X, Y = torch.meshgrid(a, a, indexing="xy")
    return torch.stack([distance * torch.tan(X).reshape(-1), distance * torch.tan(Y).reshape(-1),
                        torch.full((n_side * n_side,), distance, dtype=torch.float64)], 1).float()


def plain_forward(n_samples: int = 1000, n_sources: int = 16, seed: int = 0):
    """Plain-forward workload: (telescope, sources, values, source_type)."""
    groups, obst = davies_cotton(n_samples=n_samples, seed=seed)
    cam = SquareSensor([0.0, 0.0, 15.0], [0.0, 0.0, 0.0], 32, 30, (-0.672, 0.672, -0.63, 0.63))
    tel = Telescope(groups, obst, [cam], name="dc12m_square")
    src = point_sources_disk(n_sources, 2.5, seed + 1)
    g = torch.Generator().manual_seed(seed + 2)
    val = 0.5 + 0.5 * torch.rand(n_sources, generator=g)
    return tel, src, val, "point"


def hex_camera(n_pixels: int = 2048, pitch: float = 0.042, z: float = 15.0, edge_width: float = 0.0):
    return HexagonalSensor([0.0, 0.0, z], [0.0, 0.0, 0.0], hex_grid(n_pixels, pitch).astype(np.float32),
                           edge_width=edge_width)


def response_matrix(n_samples: int = 256, n_side: int = 64, seed: int = 0):
    """Response-matrix workload: (telescope, sources, values, source_type)."""
    groups, obst = davies_cotton(n_samples=n_samples, seed=seed)
    tel = Telescope(groups, obst, [hex_camera()], name="dc12m_hex2048")
    src = point_sources_grid(n_side, 3.0)
    return tel, src, torch.ones(src.shape[0]), "point"


def cassegrain(n_samples: int = 500, n_sources: int = 64, seed: int = 0, with_aspheric: bool = True):
    """Two-mirror Cassegrain workload: (telescope, sources, values, source_type)."""
    f = 10.0
    c1, k1 = 1.0 / (2.0 * f), -1.05
    rng = np.random.default_rng(seed)
    R = 5.0
    asph = [float(rng.normal(0.0, 1e-6) / R ** (4 * (i + 1))) for i in range(4)] if with_aspheric else []
    prim = AsphericSurface(c1, k1, asph)
    verts = hex_vertices(1.2)
    mirrors = []
    for (x, y) in hex_grid(61, 1.2):
        z0 = float(prim._sag_raw(torch.tensor(x, dtype=torch.float64), torch.tensor(y, dtype=torch.float64)))
        mirrors.append(Mirror([x, y, z0], [0.0, 0.0, 0.0], prim, PolygonAperture(verts), optical_stage=0,
                              offset=[x, y]))
    # convex hyperboloid with foci at the primary focus (z = 10) and z = -0.5,
    # vertex at z = 6 (local +z points down after the 180 deg tip)
    a = 0.5 * ((6.0 + 0.5) - (f - 6.0))
    ch = 0.5 * (f + 0.5)
    sec = AsphericSurface(-a / (ch * ch - a * a), -(ch / a) ** 2, [])
    mirrors.append(Mirror([0.0, 0.0, 6.0], [180.0, 0.0, 0.0], sec, DiskAperture(1.5), optical_stage=1))
    groups = group_mirrors(mirrors)
    key = _keys.key(seed)
    integ = MCIntegrator(n_samples)
    groups = [integ.sample_group(g, k) if g.optical_stage == 0 else g
              for g, k in zip(groups, _keys.split(key, len(groups)))]
    cam = SquareSensor([0.0, 0.0, -0.5], [0.0, 0.0, 0.0], 32, 32, (-0.45, 0.45, -0.45, 0.45))
    tel = Telescope(groups, [], [cam], name="cassegrain10m")
    src = point_sources_disk(n_sources, 1.5, seed + 1)
    return tel, src, torch.ones(n_sources), "point"


def strut_lattice(n_struts: int = 270, seed: int = 0):
    """Obstructions with a CT5-like primitive count: n_struts thin cylinders
    (radius 1-6 cm) at random between the dish and the camera, an axial
    strut, two spheres, an oriented box, a triangle and the camera box."""
    from .core import Box, Cylinder, OrientedBox, Sphere, Triangle
    from .core.transforms import euler_to_matrix
    rng = np.random.default_rng(seed + 5)
    prims = []
    for _ in range(n_struts):
        a0, a1 = rng.uniform(0, 2 * math.pi, 2)
        r0, r1 = rng.uniform(0.5, 7.5), rng.uniform(0.2, 2.0)
        z0, z1 = rng.uniform(0.5, 6.0), rng.uniform(9.0, 15.5)
        prims.append(Cylinder([r0 * math.cos(a0), r0 * math.sin(a0), z0], [r1 * math.cos(a1), r1 * math.sin(a1), z1],
                              float(rng.uniform(0.01, 0.06))))
    prims.append(Cylinder([0.0, 0.0, 2.0], [0.0, 0.0, 14.0], 0.08))  # a vertical strut on the axis
    prims += [Sphere([1.0, 0.5, 8.0], 0.4), Sphere([-2.0, 1.0, 5.0], 0.3),
              OrientedBox([0.0, -2.0, 7.0], [0.8, 0.3, 0.4], euler_to_matrix(torch.tensor([10.0, 20.0, 30.0]))),
              Triangle([-1.0, -1.0, 9.0], [1.5, -0.5, 9.5], [0.0, 1.5, 8.5]),
              Box([-0.75, -0.75, 15.0], [0.75, 0.75, 16.6])]
    return prims


def obstructed(n_samples: int = 256, n_sources: int = 16, n_struts: int = 270, seed: int = 0, pixels: int = 960):
    """Davies-Cotton dish under a lattice of struts (strut_lattice), hex
    camera, point sources: the large-obstruction-set case of the shadow
    test. Returns (telescope, sources, values, source_type)."""
    from .core import group_obstructions
    groups, _ = davies_cotton(n_samples=n_samples, seed=seed, obstructions=False)
    tel = Telescope(groups, group_obstructions(strut_lattice(n_struts, seed)), [hex_camera(pixels)],
                    name="dc380_struts")
    return tel, point_sources_disk(n_sources, 2.5, seed + 21), torch.ones(n_sources), "point"


def _first_facets(g, n: int, rot):
    """The first n facets of a sampled polygon-aperture group, with rotations `rot`."""
    return g.replace(positions=g.positions[:n], rotations=rot, offsets=g.offsets[:n], vertices=g.vertices[:n],
                     points=g.points[:n], normals=g.normals[:n], weights=g.weights[:n],
                     perturbation_delta=g.perturbation_delta[:n], perturbation_scale=g.perturbation_scale[:n])


def ragged_batch(n_instances: int = 64, n_samples: int = 256, seed: int = 0, max_facets: int = 900,
                 min_facets: int = 100, max_sources: int = 4096, pixels=(960, 2048)):
    """Ragged batch of telescope variants: (telescopes, sources, values, source_type).

    Instance i draws its facet count n uniform in [min_facets, max_facets]
    (the first n facets of one Davies-Cotton dish sampled once), a tip/tilt
    error sigma uniform in 0.2..1.0 mrad, a camera of `pixels` and a
    log-uniform source count in [1, max_sources]; sources are points at
    z = 1e10 within 2.5 deg with values U(0.5, 1)."""
    groups, obst = davies_cotton(n_facets=max_facets, tilt_sigma_mrad=0.0, n_samples=n_samples, seed=seed)
    if len(groups) != 1:
        raise ValueError("the Davies-Cotton dish is expected to form one mirror group")
    g = groups[0]
    rng = np.random.default_rng(seed + 101)
    cams = {p: hex_camera(p) for p in pixels}
    tels, srcs, vals = [], [], []
    for i in range(n_instances):
        n = int(rng.integers(min_facets, max_facets + 1))
        S = int(min(max_sources, max(1, round(math.exp(rng.uniform(0.0, math.log(max_sources)))))))
        P = int(pixels[int(rng.integers(0, len(pixels)))])
        sig_deg = math.degrees(float(rng.uniform(0.2, 1.0)) * 1e-3)
        rot = g.rotations[:n].clone()
        rot[:, :2] += torch.from_numpy(rng.standard_normal((n, 2))).float() * sig_deg
        tels.append(Telescope([_first_facets(g, n, rot)], obst, [cams[P]], name=f"dc_variant{i}_{n}f_{P}px"))
        srcs.append(point_sources_disk(S, 2.5, seed + 1000 + i))
        vals.append(0.5 + 0.5 * torch.from_numpy(rng.random(S)).float())
    return tels, srcs, vals, "point"
