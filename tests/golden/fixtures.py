"""Rebuild a golden fixture (tests/golden/*.npz, written by make_golden.py
from the reference itself) as an iactrace_gb300 Telescope fed the same
sampled arrays."""
from __future__ import annotations

import json
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("ct3_point", "cass_parallel", "dc_mixed", "seg_cassegrain", "tilted_cams")


def path(case: str, kind: str) -> str:
    return os.path.join(HERE, f"{case}_{kind}.npz")


def load(case: str, kind: str):
    return dict(np.load(path(case, kind), allow_pickle=False))


def telescope(fx):
    from iactrace_gb300 import (DifferentiableHexagonalSensor, DifferentiableSquareSensor, HexagonalSensor,
                                SquareSensor, Telescope)
    from iactrace_gb300.core import (AsphericSurface, BoxGroup, CylinderGroup, OrientedBoxGroup, SphereGroup,
                                     TriangleGroup)
    from iactrace_gb300.telescope import AsphericDiskMirrorGroup, AsphericPolygonMirrorGroup

    f32 = lambda k: torch.from_numpy(np.ascontiguousarray(fx[k].astype(np.float32)))
    F = fx["prim_positions"].shape[0]
    prim = AsphericDiskMirrorGroup(f32("prim_positions"), f32("prim_rotations"), AsphericSurface(0.0, 0.0, []),
                                   torch.ones(F), optical_stage=0)
    prim = prim.replace(points=f32("prim_points"), normals=f32("prim_normals"),
                        perturbation_delta=f32("prim_perturbation_delta"), weights=f32("prim_weights"),
                        perturbation_scale=f32("prim_perturbation_scale"))
    groups = [prim]
    for r in json.loads(str(fx["stage_mirrors_json"])):
        surf = AsphericSurface(r["curvature"], r["conic"], r["aspheric"])
        if "radius" in r:
            g = AsphericDiskMirrorGroup([r["pos"]], [r["rot"]], surf, [r["radius"]], r["stage"], [r["offset"]])
        else:
            g = AsphericPolygonMirrorGroup([r["pos"]], [r["rot"]], surf, [r["vertices"]], r["stage"], [r["offset"]])
        groups.append(g)
    obst = []
    for k, cls in (("cyl", CylinderGroup), ("box", BoxGroup), ("sph", SphereGroup), ("obox", OrientedBoxGroup),
                   ("tri", TriangleGroup)):
        if "obst_" + k in fx:
            t = f32("obst_" + k)
            if k == "cyl":
                obst.append(cls(p1=t[:, :3], p2=t[:, 3:6], r=t[:, 6]))
            elif k == "box":
                obst.append(cls(p1=t[:, :3], p2=t[:, 3:6]))
            elif k == "sph":
                obst.append(cls(centers=t[:, :3], radii=t[:, 3]))
            elif k == "obox":
                obst.append(cls(centers=t[:, :3], half_extents=t[:, 3:6], rotations=t[:, 6:]))
            else:
                obst.append(cls(v0=t[:, :3], v1=t[:, 3:6], v2=t[:, 6:9]))
    sensors = []
    for i, d in enumerate(json.loads(str(fx["sensors_json"]))):
        c = d["class"]
        if "Square" in c:
            b = (d["x0"], d["x0"] + d["dx"] * d["width"], d["y0"], d["y0"] + d["dy"] * d["height"])
            if c.startswith("Differentiable"):
                s = DifferentiableSquareSensor(d["position"], d["rotation"], d["width"], d["height"], b,
                                               sigma=d["sigma"], kernel_size=d["kernel_size"])
            else:
                s = SquareSensor(d["position"], d["rotation"], d["width"], d["height"], b, edge_width=d["edge_width"])
            # the reference's own float constants (bounds -> x0, dx) verbatim
            s.x0, s.y0, s.dx, s.dy = d["x0"], d["y0"], d["dx"], d["dy"]
        else:
            centers = fx[f"hex_centers_{i}"]
            if c.startswith("Differentiable"):
                s = DifferentiableHexagonalSensor(d["position"], d["rotation"], centers, sigma=d["sigma"],
                                                  kernel_size=d["kernel_size"])
            else:
                s = HexagonalSensor(d["position"], d["rotation"], centers, edge_width=d["edge_width"])
            # the grid constants the reference derived in this precision: its
            # float32 and float64 runs can detect different (60-degree
            # equivalent) grid frames and build different lookup tables
            s.hex_size, s.hex_inradius, s.grid_rotation = d["hex_size"], d["hex_inradius"], d["grid_rotation"]
            s.grid_offset = tuple(d["grid_offset"])
            s.q_min, s.r_min = d["q_min"], d["r_min"]
            s.lookup_table = torch.from_numpy(np.ascontiguousarray(fx[f"hex_table_{i}"].astype(np.int32)))
        sensors.append(s)
    return Telescope(groups, obst, sensors, name="golden")


def inputs(fx):
    return (torch.from_numpy(fx["sources"].astype(np.float32)), torch.from_numpy(fx["values"].astype(np.float32)),
            str(fx["source_type"]))


def sensor_ids(fx):
    return sorted(int(k.split("_")[1]) for k in fx if k.startswith("image_") and k.endswith("_shape"))


def image(fx, si):
    shape = tuple(int(v) for v in fx[f"image_{si}_shape"])
    if f"image_{si}" in fx:
        return fx[f"image_{si}"].reshape(shape)
    out = np.zeros(int(np.prod(shape)), fx[f"image_{si}_val"].dtype)
    out[fx[f"image_{si}_idx"]] = fx[f"image_{si}_val"]
    return out.reshape(shape)
