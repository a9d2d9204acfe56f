#!/usr/bin/env python
"""Generate the golden fixtures of the render path from the reference itself.

Runs GerritRo/iactrace's own Python source (a checkout named by the
IACTRACE_REFERENCE environment variable) on the numpy stand-in for jax/equinox in tests/golden/jaxshim (JAX cannot be
installed here), builds a few small scenes with the reference's API,
renders them with the reference's render / render_debug /
render_response_matrix, and stores inputs and outputs as .npz files beside
this script:

  <case>_f32.npz   the reference in float32 (JAX's default, x64 off)
  <case>_f64.npz   the same scene and the same sampled arrays, rendered by
                   the reference with float64 arithmetic (JAX x64 mode)

Cases:
  ct3_point      configs/HESS/CT3.yaml through the reference loader
                 (MCIntegrator(8), roughness 24"), 2 point sources at 1e10 m,
                 hex camera (sensor 0) and the square lid (sensor 1)
  cass_parallel  a two-mirror Cassegrain (6 disk segments on a paraboloid,
                 hyperbolic secondary, aspheric terms on both), 4 parallel
                 sources, square camera
  dc_mixed       a 19-facet Davies-Cotton dish with every obstruction kind
                 (cylinder, box, sphere, oriented box, triangle), point
                 sources at 1 km, square + hex cameras with edge bands and
                 the two soft-splat sensors
  tilted_cams    the 19-facet dish imaged by tilted and rolled square and
                 hexagonal cameras (general plane-hit form; hexagon centres
                 rotated by 10 deg), hard with edge bands and soft
  seg_cassegrain the Cassegrain primary with a segmented secondary (three
                 disk segments and a central hexagon cut from one
                 hyperboloid: two mirror groups in stage 1), 4 parallel
                 sources, square camera

The per-ray sensor-plane hits and values of the first sensor are stored
(debug_pts, debug_vals), and for a hard first sensor also the pixel id the
reference's own accumulate gives each hit (debug_pix, -1 for none); for
scenes with one later stage, the stage mirror each ray's closest hit takes
(debug_hit_mirror, -1 for none).

Usage: IACTRACE_REFERENCE=<checkout of GerritRo/iactrace> python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import math
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("IACTRACE_REFERENCE", "")
if not os.path.isdir(os.path.join(REF, "iactrace")):
    sys.exit("set IACTRACE_REFERENCE to a checkout of GerritRo/iactrace (the directory holding iactrace/)")
sys.path[:0] = [os.path.join(HERE, "jaxshim"), REF]
X64 = os.environ.get("JAXSHIM_X64") == "1"

import numpy as np  # noqa: E402

import equinox as eqx  # noqa: E402
import jax  # noqa: E402
import jax.numpy as jnp  # noqa: E402
from iactrace import MCIntegrator, load_telescope  # noqa: E402
from iactrace.core import (AsphericSurface, Box, Cylinder, DiskAperture, OrientedBox, PolygonAperture,  # noqa: E402
                           Sphere, Triangle, euler_to_matrix, group_obstructions, render, render_debug,
                           render_response_matrix)
from iactrace.sensors.hexagonal import DifferentiableHexagonalSensor, HexagonalSensor  # noqa: E402
from iactrace.sensors.square import DifferentiableSquareSensor, SquareSensor  # noqa: E402
from iactrace.telescope import Mirror, Telescope, group_mirrors  # noqa: E402

FT = np.float64 if X64 else np.float32
SUFFIX = "f64" if X64 else "f32"


def A(x):
    return np.asarray(x)


# ------------------------------------------------------------------ scenes

def scene_ct3():
    tel = load_telescope(os.path.join(REF, "configs/HESS/CT3.yaml"), MCIntegrator(8), jax.random.key(0))
    tel = tel.apply_roughness(24.0)
    src = jnp.array([[0.0, 0.0, 1e10], [1.2e8, -0.7e8, 1e10]])
    val = jnp.array([1.0, 0.75])
    return tel, src, val, "point", [0, 1]


def scene_cassegrain(sec_radius=1.2, theta_deg=(0.0, 0.4, 0.7, 0.9)):
    f = 10.0
    prim = AsphericSurface(curvature=1.0 / (2 * f), conic=-1.0, aspheric=jnp.array([2e-6, -1e-8]))
    # hyperbolic secondary: foci at the primary focus and 0.5 m behind the vertex
    a, ch = 1.25, 5.25
    sec = AsphericSurface(curvature=-a / (ch * ch - a * a), conic=-(ch / a) ** 2, aspheric=jnp.array([1e-4]))
    mirrors = []
    for k in range(6):
        ang = math.radians(60 * k + 15)
        x, y = 2.2 * math.cos(ang), 2.2 * math.sin(ang)
        z0 = (x * x + y * y) / (4 * f)
        mirrors.append(Mirror(position=jnp.array([x, y, z0]), rotation=jnp.array([0.0, 0.0, 0.0]), surface=prim,
                              aperture=DiskAperture(0.9), offset=jnp.array([x, y]), optical_stage=0))
    mirrors.append(Mirror(position=jnp.array([0.0, 0.0, 6.0]), rotation=jnp.array([180.0, 0.0, 0.0]), surface=sec,
                          aperture=DiskAperture(sec_radius), optical_stage=1))
    groups = group_mirrors(mirrors)
    key = jax.random.key(7)
    integ = MCIntegrator(16)
    out = []
    for g in groups:
        if g.optical_stage == 0:
            key, sub = jax.random.split(key)
            out.append(integ.sample_group(g, sub))
        else:
            out.append(g)
    cam = SquareSensor(position=[0.0, 0.0, -0.5], rotation=[0.0, 0.0, 0.0], width=24, height=24,
                       bounds=(-0.3, 0.3, -0.3, 0.3))
    tel = Telescope(mirror_groups=out, obstruction_groups=[], sensors=[cam], name="cass")
    th = np.radians(list(theta_deg))
    ph = np.radians([0.0, 30.0, 200.0, 300.0])
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)], 1)
    return tel, jnp.array(d), jnp.array([1.0, 2.0, 0.5, 1.5]), "parallel", [0]


def scene_seg_cassegrain():
    """The Cassegrain primary with a segmented secondary: three disk
    segments around the axis and a central hexagonal one, cut from one
    hyperboloid (two mirror groups in stage 1), so the closest-hit choice
    between mirrors of a stage decides every ray; 4 parallel sources."""
    base, _, _, _, _ = scene_cassegrain()
    f = 10.0
    a, ch = 1.25, 5.25
    sec = AsphericSurface(curvature=-a / (ch * ch - a * a), conic=-(ch / a) ** 2, aspheric=jnp.array([1e-4]))
    segs = []
    for k in range(3):
        ang = math.radians(120 * k + 30)
        x0, y0 = 0.7 * math.cos(ang), 0.7 * math.sin(ang)
        z0 = float(A(sec._sag_raw(jnp.array(x0), jnp.array(y0))))
        # the parent's frame is tipped by 180 deg (local y and z flip in the world)
        segs.append(Mirror(position=jnp.array([x0, -y0, 6.0 - z0]), rotation=jnp.array([180.0, 0.0, 0.0]),
                           surface=sec, aperture=DiskAperture(0.58), offset=jnp.array([x0, y0]), optical_stage=1))
    rc = 0.34
    hexv = [[rc * math.cos(math.radians(60 * k)), rc * math.sin(math.radians(60 * k))] for k in range(6)]
    segs.append(Mirror(position=jnp.array([0.0, 0.0, 6.0]), rotation=jnp.array([180.0, 0.0, 0.0]), surface=sec,
                       aperture=PolygonAperture(jnp.array(hexv)), optical_stage=1))
    prim = [g for g in base.mirror_groups if g.optical_stage == 0]
    tel = Telescope(mirror_groups=prim + group_mirrors(segs), obstruction_groups=[], sensors=base.sensors,
                    name="cass_segmented")
    th = np.radians([0.0, 0.25, 0.45, 0.6])
    ph = np.radians([0.0, 75.0, 160.0, 250.0])
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)], 1)
    return tel, jnp.array(d), jnp.array([1.0, 2.0, 0.5, 1.5]), "parallel", [0]


def scene_tilted_cams():
    """The 19-facet Davies-Cotton dish of dc_mixed (two cylinders and the
    camera box as obstructions) imaged by tilted and rolled cameras: the
    sensor frame is not the world's, so the plane hit takes the general
    form, and the hexagonal camera's centres are rotated by 10 deg (a grid
    rotation the detection must find); hard sensors with edge bands and the
    two soft sensors; point sources at 1 km."""
    base, src, val, st, _ = scene_dc_mixed()
    obst = group_obstructions([
        Cylinder([1.8, 1.0, 0.5], [0.4, 0.2, 8.3], 0.04),
        Cylinder([-1.8, 1.0, 0.5], [-0.4, 0.2, 8.3], 0.04),
        Box([-0.35, -0.3, 8.0], [0.35, 0.3, 8.9]),
    ])
    f = 8.0
    c, sn = math.cos(math.radians(10.0)), math.sin(math.radians(10.0))
    hp = _hex_points(91, 0.03)
    hex_centers = np.stack([c * hp[:, 0] - sn * hp[:, 1], sn * hp[:, 0] + c * hp[:, 1]], 1)
    rs, rh = [2.0, -1.5, 25.0], [-1.5, 1.0, 40.0]
    sensors = [
        SquareSensor(position=[0.01, -0.02, f], rotation=rs, width=20, height=16, bounds=(-0.3, 0.3, -0.24, 0.24),
                     edge_width=0.002),
        HexagonalSensor(position=[-0.01, 0.015, f], rotation=rh, hex_centers=jnp.array(hex_centers), edge_width=0.001),
        DifferentiableSquareSensor(position=[0.01, -0.02, f], rotation=rs, width=20, height=16,
                                   bounds=(-0.3, 0.3, -0.24, 0.24), sigma=0.4, kernel_size=2),
        DifferentiableHexagonalSensor(position=[-0.01, 0.015, f], rotation=rh, hex_centers=jnp.array(hex_centers),
                                      sigma=0.5, kernel_size=1),
    ]
    tel = Telescope(mirror_groups=base.mirror_groups, obstruction_groups=obst, sensors=sensors, name="dc19_tilted")
    return tel, src, val, st, [0, 1, 2, 3]


def _hex_points(n, pitch):
    pts = []
    for q in range(-6, 7):
        for r in range(-6, 7):
            pts.append((pitch * (q + r / 2.0), pitch * math.sqrt(3) / 2.0 * r))
    pts = np.array(pts)
    order = np.lexsort((np.round(np.arctan2(pts[:, 1], pts[:, 0]), 9), np.round(np.hypot(pts[:, 0], pts[:, 1]), 9)))
    return pts[order[:n]]


def scene_dc_mixed():
    f = 8.0
    surf = AsphericSurface(curvature=1.0 / (2 * f), conic=0.0, aspheric=jnp.array([]))
    rc = 0.5 / math.sqrt(3)
    verts = [[rc * math.cos(math.radians(90 + 60 * k)), rc * math.sin(math.radians(90 + 60 * k))] for k in range(6)]
    rng = np.random.default_rng(3)
    mirrors = []
    for (x, y) in _hex_points(19, 0.5):
        z = f - math.sqrt(f * f - x * x - y * y)
        n = np.array([-x, -y, 2 * f - z])
        n /= np.linalg.norm(n)
        rot = [-math.degrees(math.asin(n[1])) + 0.03 * rng.standard_normal(),
               math.degrees(math.atan2(n[0], n[2])) + 0.03 * rng.standard_normal(), 0.0]
        mirrors.append(Mirror(position=jnp.array([x, y, z]), rotation=jnp.array(rot), surface=surf,
                              aperture=PolygonAperture(jnp.array(verts)), optical_stage=0))
    groups = group_mirrors(mirrors)
    key = jax.random.key(11)
    integ = MCIntegrator(12)
    sampled = []
    for g in groups:
        key, sub = jax.random.split(key)
        sampled.append(integ.sample_group(g, sub))
    obst = group_obstructions([
        Cylinder([1.8, 1.0, 0.5], [0.4, 0.2, 8.3], 0.04),
        Cylinder([-1.8, 1.0, 0.5], [-0.4, 0.2, 8.3], 0.04),
        Box([-0.35, -0.3, 8.0], [0.35, 0.3, 8.9]),
        Sphere([0.6, -0.5, 5.0], 0.15),
        OrientedBox([-0.5, -0.9, 6.0], [0.3, 0.1, 0.2], euler_to_matrix(jnp.array([10.0, 25.0, 40.0]))),
        Triangle([0.2, 0.9, 4.0], [0.9, 1.4, 4.5], [-0.2, 1.5, 4.2]),
    ])
    hex_centers = _hex_points(91, 0.03)
    sensors = [
        SquareSensor(position=[0.0, 0.0, f], rotation=[0.0, 0.0, 0.0], width=20, height=16,
                     bounds=(-0.3, 0.3, -0.24, 0.24), edge_width=0.002),
        HexagonalSensor(position=[0.0, 0.0, f], rotation=[0.0, 0.0, 0.0], hex_centers=jnp.array(hex_centers),
                        edge_width=0.001),
        DifferentiableSquareSensor(position=[0.0, 0.0, f], rotation=[0.0, 0.0, 0.0], width=20, height=16,
                                   bounds=(-0.3, 0.3, -0.24, 0.24), sigma=0.4, kernel_size=2),
        DifferentiableHexagonalSensor(position=[0.0, 0.0, f], rotation=[0.0, 0.0, 0.0],
                                      hex_centers=jnp.array(hex_centers), sigma=0.5, kernel_size=1),
    ]
    tel = Telescope(mirror_groups=sampled, obstruction_groups=obst, sensors=sensors, name="dc19")
    src = jnp.array([[0.0, 0.0, 1000.0], [15.0, -8.0, 1000.0], [-20.0, 10.0, 1000.0]])
    return tel, src, jnp.array([1.0, 0.6, 0.8]), "point", [0, 1, 2, 3]


CASES = {"ct3_point": scene_ct3, "cass_parallel": scene_cassegrain, "dc_mixed": scene_dc_mixed,
         "seg_cassegrain": scene_seg_cassegrain, "tilted_cams": scene_tilted_cams}


# --------------------------------------------------------------- recording

def scene_arrays(tel):
    """Everything the render reads, in plain arrays."""
    out = {}
    prim = [g for g in tel.mirror_groups if g.optical_stage == 0]
    for name in ("positions", "rotations", "perturbation_scale", "points", "normals", "perturbation_delta",
                 "weights"):
        out["prim_" + name] = np.concatenate([A(getattr(g, name)) for g in prim])
    later = sorted([g for g in tel.mirror_groups if g.optical_stage != 0], key=lambda g: g.optical_stage)
    recs = []
    for g in later:
        for i in range(len(g)):
            r = {"stage": int(g.optical_stage), "pos": A(g.positions[i]).tolist(), "rot": A(g.rotations[i]).tolist(),
                 "offset": A(g.offsets[i]).tolist(), "curvature": float(g.curvature), "conic": float(g.conic),
                 "aspheric": A(g.aspheric).tolist()}
            if hasattr(g, "radii"):
                r["radius"] = float(A(g.radii[i]))
            else:
                r["vertices"] = A(g.vertices[i]).tolist()
            recs.append(r)
    out["stage_mirrors_json"] = np.array(json.dumps(recs))
    tabs = {}
    for g in (tel.obstruction_groups or []):
        kind = type(g).__name__
        if kind == "CylinderGroup":
            tabs.setdefault("cyl", []).append(np.concatenate([A(g.p1), A(g.p2), A(g.r)[:, None]], 1))
        elif kind == "BoxGroup":
            tabs.setdefault("box", []).append(np.concatenate([A(g.p1), A(g.p2)], 1))
        elif kind == "SphereGroup":
            tabs.setdefault("sph", []).append(np.concatenate([A(g.centers), A(g.radii)[:, None]], 1))
        elif kind == "OrientedBoxGroup":
            tabs.setdefault("obox", []).append(np.concatenate([A(g.centers), A(g.half_extents),
                                                               A(g.rotations).reshape(-1, 9)], 1))
        elif kind == "TriangleGroup":
            tabs.setdefault("tri", []).append(np.concatenate([A(g.v0), A(g.v1), A(g.v2)], 1))
    for k, v in tabs.items():
        out["obst_" + k] = np.concatenate(v)
    sens = []
    for s in tel.sensors:
        d = {"class": type(s).__name__, "position": A(s.position).tolist(), "rotation": A(s.rotation).tolist()}
        if "Square" in d["class"]:
            d.update(width=s.width, height=s.height, x0=s.x0, y0=s.y0, dx=s.dx, dy=s.dy)
            d["edge_width"] = getattr(s, "edge_width", 0.0)
        else:
            d.update(hex_size=s.hex_size, hex_inradius=s.hex_inradius, grid_rotation=s.grid_rotation,
                     grid_offset=list(s.grid_offset), q_min=s.q_min, r_min=s.r_min, n_pixels=s.n_pixels)
            d["edge_width"] = getattr(s, "edge_width", 0.0)
            out[f"hex_centers_{len(sens)}"] = A(s.hex_centers)
            out[f"hex_table_{len(sens)}"] = A(s.lookup_table)
        if "Differentiable" in d["class"]:
            d.update(sigma=s.sigma, kernel_size=int(getattr(s, "kernel_size", 0) or (
                int(np.max(np.abs(A(s.neighbor_offsets_q)))) if hasattr(s, "neighbor_offsets_q") else 0)))
        sens.append(d)
    out["sensors_json"] = np.array(json.dumps(sens))
    return out


def inject_samples(tel, f32_fixture):
    """Feed the float32 run's sampled arrays (as float64) into the x64 scene."""
    prim_idx = [i for i, g in enumerate(tel.mirror_groups) if g.optical_stage == 0]
    groups = list(tel.mirror_groups)
    start = 0
    for i in prim_idx:
        g = groups[i]
        n = len(g)
        sl = slice(start, start + n)
        start += n
        g = eqx.tree_at(lambda q: (q.points, q.normals, q.perturbation_delta, q.weights, q.positions, q.rotations,
                                   q.perturbation_scale), g,
                        tuple(jnp.array(f32_fixture["prim_" + k][sl].astype(np.float64))
                              for k in ("points", "normals", "perturbation_delta", "weights", "positions",
                                        "rotations", "perturbation_scale")))
        groups[i] = g
    return eqx.tree_at(lambda t: t.mirror_groups, tel, groups)


def ref_pixel_ids(sensor, pts):
    """Per-ray pixel ids decided by the reference's own hard accumulate
    (sensors/square.py:66-91, sensors/hexagonal.py:174-194): each hit alone
    with value 1; -1 where it lands in no pixel (out of bounds, no table
    entry, inside the edge band)."""
    out = np.full(len(pts), -1, np.int32)
    for i in range(len(pts)):
        img = A(sensor.accumulate(jnp.array(pts[i:i + 1, 0]), jnp.array(pts[i:i + 1, 1]),
                                  jnp.ones(1, dtype=pts.dtype))).reshape(-1)
        nz = np.flatnonzero(img)
        if nz.size:
            out[i] = nz[0]
    return out


def ref_hit_mirror(tel, src, st):
    """Per ray (order facet, source, sample) the stage-1 mirror that the
    reference's closest-hit choice takes (core/render.py:44-115): each
    mirror's t from the reference's own _intersect_group on a one-mirror
    group, the first of the minimal t in the scene's group and mirror order
    (argmin within a group, strict `<` across groups), -1 without a hit
    (t >= 1e10). Scenes with one later stage."""
    from iactrace.core.reflection import reflect
    from iactrace.core.render import _get_stages, _intersect_group
    stages = _get_stages(tel.mirror_groups)
    assert sorted(stages) == [0, 1]
    data = [g.transform_to_world() for g in stages[0]]
    tp_all = np.concatenate([A(d[0]) for d in data])
    tn_all = np.concatenate([A(d[1]) for d in data])
    singles = []
    for g in stages[1]:
        names = ["positions", "rotations", "offsets"] + (["radii"] if hasattr(g, "radii") else ["vertices"])
        for j in range(len(g)):
            singles.append(eqx.tree_at(lambda q: tuple(getattr(q, n) for n in names), g,
                                       tuple(getattr(g, n)[j:j + 1] for n in names)))
    srcs = A(src)
    out = []
    for f in range(tp_all.shape[0]):
        tp, tn = jnp.array(tp_all[f]), jnp.array(tn_all[f])
        for s in range(srcs.shape[0]):
            if st == "point":
                w = tp_all[f] - srcs[s][None, :]
                d = jnp.array(w / np.linalg.norm(w, axis=-1, keepdims=True))
            else:
                d = jnp.array(np.broadcast_to(srcs[s], tp_all[f].shape))
            r = jax.vmap(reflect)(d, tn)[0]
            T = np.stack([A(_intersect_group(tp, r, g1)[0]) for g1 in singles])
            best = np.argmin(T, axis=0)
            out.append(np.where(T.min(axis=0) < 1e10, best, -1))
    return np.concatenate(out).astype(np.int32)


def run_case(name):
    t0 = time.time()
    tel, src, val, st, sensors = CASES[name]()
    path32 = os.path.join(HERE, f"{name}_f32.npz")
    if X64:
        tel = inject_samples(tel, np.load(path32))
        src = jnp.array(A(src).astype(np.float64))
        val = jnp.array(A(val).astype(np.float64))
    rec = scene_arrays(tel)
    rec["sources"], rec["values"], rec["source_type"] = A(src), A(val), np.array(st)
    for si in sensors:
        shape = tel.sensors[si].get_accumulator_shape()
        img = A(render(tel, src, val, st, si))
        if img.size > 20000:  # large images: non-zero entries only
            nz = np.flatnonzero(img.reshape(-1))
            rec[f"image_{si}_idx"], rec[f"image_{si}_val"] = nz.astype(np.int32), img.reshape(-1)[nz]
        else:
            rec[f"image_{si}"] = img
        rec[f"image_{si}_shape"] = np.array(shape)
        if img.size <= 20000:
            rec[f"response_{si}"] = A(render_response_matrix(tel, src, val, st, si))
        if si == sensors[0]:
            pts, vals = render_debug(tel, src, val, st, si)
            rec["debug_pts"], rec["debug_vals"] = A(pts), A(vals)
            if "Differentiable" not in type(tel.sensors[si]).__name__:
                rec["debug_pix"] = ref_pixel_ids(tel.sensors[si], A(pts))
            if sorted({g.optical_stage for g in tel.mirror_groups}) == [0, 1]:
                rec["debug_hit_mirror"] = ref_hit_mirror(tel, src, st)
    out = os.path.join(HERE, f"{name}_{SUFFIX}.npz")
    np.savez_compressed(out, **rec)
    print(f"{name} ({SUFFIX}): {time.time() - t0:.1f} s -> {os.path.basename(out)} "
          f"({os.path.getsize(out) / 1024:.0f} KiB)", flush=True)


def main():
    names = [a for a in sys.argv[1:] if not a.startswith("-")] or list(CASES)
    for n in names:
        run_case(n)
    if not X64 and "--no-x64" not in sys.argv:
        env = dict(os.environ, JAXSHIM_X64="1")
        subprocess.run([sys.executable, __file__, *names], env=env, check=True)


if __name__ == "__main__":
    main()
