#!/usr/bin/env python
"""Scene-construction fixtures from the reference itself: what
GerritRo/iactrace's own loader and editors produce, for the host-side
parity tests (tests/test_scene_parity.py).

Runs the reference's Python source (a checkout named by the
IACTRACE_REFERENCE environment variable) on the numpy stand-in for
jax/equinox/pyyaml (tests/golden/jaxshim) in float32 (JAX's default):

  loader_CT3.npz, loader_CT5.npz
      load_telescope(configs/HESS/<name>.yaml, MCIntegrator(2), key(0))
      (io/yaml_loader.py:29-171): every deterministic field of the result:
      the mirror-group partition (telescope/mirrors.py:232-313: class,
      stage, surface curvature / conic / aspheric terms, positions,
      rotations, offsets, radii or polygon vertices), the obstruction groups
      (core/obstructions.py:258-277: class and tables), and the sensors
      (class, pose, pixel geometry, hexagon grid constants and lookup table).
      The sampled arrays are not stored: their random streams are the
      stand-in's, not threefry's.
  editors_CT3.npz
      the editors of telescope/operations.py applied to the loaded CT3:
      apply_roughness(24"), apply_roughness_to_group(0, 12"),
      scale_mirror_weights (scalar and per mirror), set_mirror_rotations,
      set_mirror_positions, focus, apply_misalignment_to_group(0, 20", 35")
      and apply_displacement_to_group(0, 3 mm) with the unit-normal draws
      the reference's own function made (so a test can feed the same draws
      to another implementation and compare the deterministic part).

Usage: IACTRACE_REFERENCE=<checkout> python tests/golden/make_scene_golden.py
"""
from __future__ import annotations

import json
import os
import sys

os.environ.pop("JAXSHIM_X64", None)
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import make_golden as MG  # noqa: E402  (imports the reference on the stand-in, float32)

jax, jnp = MG.jax, MG.jnp
A = MG.A
ref_ops = __import__("iactrace.telescope.operations", fromlist=["operations"])


def config_path(name):
    return os.path.join(MG.REF, "configs", "HESS", f"{name}.yaml")


def record_telescope(tel, prefix=""):
    rec = {}
    groups = []
    for i, g in enumerate(tel.mirror_groups):
        d = {"class": type(g).__name__, "stage": int(g.optical_stage), "curvature": float(g.curvature),
             "conic": float(g.conic), "n": len(g)}
        groups.append(d)
        for k in ("positions", "rotations", "offsets", "aspheric", "perturbation_scale"):
            rec[f"{prefix}g{i}_{k}"] = A(getattr(g, k))
        rec[f"{prefix}g{i}_" + ("radii" if hasattr(g, "radii") else "vertices")] = \
            A(g.radii if hasattr(g, "radii") else g.vertices)
    obst = []
    fields = {"CylinderGroup": ("p1", "p2", "r"), "BoxGroup": ("p1", "p2"), "SphereGroup": ("centers", "radii"),
              "OrientedBoxGroup": ("centers", "half_extents", "rotations"), "TriangleGroup": ("v0", "v1", "v2")}
    for i, g in enumerate(tel.obstruction_groups or []):
        cls = type(g).__name__
        obst.append(cls)
        for k in fields[cls]:
            rec[f"{prefix}o{i}_{k}"] = A(getattr(g, k))
    sensors = []
    for i, s in enumerate(tel.sensors):
        d = {"class": type(s).__name__, "edge_width": float(getattr(s, "edge_width", 0.0))}
        rec[f"{prefix}s{i}_position"], rec[f"{prefix}s{i}_rotation"] = A(s.position), A(s.rotation)
        if "Square" in d["class"]:
            d.update(width=s.width, height=s.height, x0=s.x0, y0=s.y0, dx=s.dx, dy=s.dy)
        else:
            d.update(hex_size=s.hex_size, hex_inradius=s.hex_inradius, grid_rotation=s.grid_rotation,
                     grid_offset=list(s.grid_offset), q_min=s.q_min, r_min=s.r_min, n_pixels=s.n_pixels)
            rec[f"{prefix}s{i}_hex_centers"] = A(s.hex_centers)
            rec[f"{prefix}s{i}_lookup_table"] = A(s.lookup_table)
        sensors.append(d)
    rec[f"{prefix}meta"] = np.array(json.dumps({"name": tel.name, "groups": groups, "obstructions": obst,
                                                "sensors": sensors}))
    return rec


def loader_fixture(name):
    tel = MG.load_telescope(config_path(name), MG.MCIntegrator(2), jax.random.key(0))
    out = os.path.join(HERE, f"loader_{name}.npz")
    np.savez_compressed(out, **record_telescope(tel))
    print(f"loader {name}: {len(tel.mirror_groups)} mirror groups, "
          f"{len(tel.obstruction_groups or [])} obstruction groups, {len(tel.sensors)} sensors -> "
          f"{os.path.basename(out)} ({os.path.getsize(out) / 1024:.0f} KiB)", flush=True)
    return tel


def editors_fixture(tel):
    rec = {"weights0": A(tel.mirror_groups[0].weights), "rotations0": A(tel.mirror_groups[0].rotations),
           "positions0": A(tel.mirror_groups[0].positions), "sensor_position0": A(tel.sensors[0].position)}
    n = len(tel.mirror_groups[0])
    t = ref_ops.apply_roughness(tel, 24.0)
    rec["roughness_scale"] = np.stack([A(g.perturbation_scale) for g in t.mirror_groups[:1]])
    t = ref_ops.apply_roughness_to_group(tel, 0, 12.0)
    rec["roughness_group_scale"] = A(t.mirror_groups[0].perturbation_scale)
    rec["weights_scalar"] = A(ref_ops.scale_mirror_weights(tel, 0, 0.8).mirror_groups[0].weights)
    factors = np.linspace(0.5, 1.0, n).astype(np.float32)
    rec["weight_factors"] = factors
    rec["weights_per_mirror"] = A(ref_ops.scale_mirror_weights(tel, 0, jnp.array(factors)).mirror_groups[0].weights)
    new_rot = A(tel.mirror_groups[0].rotations) + np.float32(0.01)
    rec["set_rotations"] = A(ref_ops.set_mirror_rotations(tel, 0, jnp.array(new_rot)).mirror_groups[0].rotations)
    new_pos = A(tel.mirror_groups[0].positions) * np.float32(1.001)
    rec["set_positions"] = A(ref_ops.set_mirror_positions(tel, 0, jnp.array(new_pos)).mirror_groups[0].positions)
    rec["focus_position"] = A(ref_ops.focus(tel, 0.01, 0).sensors[0].position)
    # the draws the reference's own functions make: the same key splits as
    # telescope/operations.py:185-188 and :221
    key = jax.random.key(5)
    k1, k2 = jax.random.split(key)
    rec["misalign_z_h"] = A(jax.random.normal(k1, shape=(n,)))
    rec["misalign_z_v"] = A(jax.random.normal(k2, shape=(n,)))
    rec["misalign_rotations"] = A(ref_ops.apply_misalignment_to_group(tel, 0, 20.0, 35.0, key).mirror_groups[0].rotations)
    key = jax.random.key(6)
    rec["displace_z"] = A(jax.random.normal(key, shape=(n,)))
    rec["displace_positions"] = A(ref_ops.apply_displacement_to_group(tel, 0, 0.003, key).mirror_groups[0].positions)
    out = os.path.join(HERE, "editors_CT3.npz")
    np.savez_compressed(out, **rec)
    print(f"editors: -> {os.path.basename(out)} ({os.path.getsize(out) / 1024:.0f} KiB)", flush=True)


def main():
    ct3 = loader_fixture("CT3")
    loader_fixture("CT5")
    editors_fixture(ct3)


if __name__ == "__main__":
    main()
