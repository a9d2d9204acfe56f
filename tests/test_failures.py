"""Failure detection on the host (no GPU fault is ever provoked): bad scene
files, NaN / Inf parameters and bad indices are rejected before anything is
launched; the C ABI returns status codes (tests/test_native_abi.py)."""
from __future__ import annotations

import math

import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300 import Telescope, workloads as W
from iactrace_gb300.core import Cylinder, Sphere, group_obstructions
from iactrace_gb300.core.scene import pack_scene

YAML = """
telescope:
  name: tiny
mirror_templates:
  facet:
    surface:
      curvature: 0.0333
      conic: 0.0
mirrors:
  - template: facet
    position: [0.0, 0.0, 0.0]
    orientation: [0.0, 0.0, 0.0]
    aperture:
      type: circular
      radius: 0.3
obstructions:
  - type: %s
    p1: [0.0, 0.0, 1.0]
    p2: [0.0, 0.0, 2.0]
    r: 0.1
sensors:
  - type: square
    position: [0.0, 0.0, 15.0]
    orientation: [0.0, 0.0, 0.0]
    width: 4
    height: 4
    bounds: [-0.1, 0.1, -0.1, 0.1]
"""

def test_unknown_obstruction_type_in_scene_file(tmp_path):
    f = tmp_path / "bad.yaml"
    f.write_text(YAML % "pyramid")
    with pytest.raises(ValueError, match="Unknown obstruction type"):
        it.load_telescope(str(f), it.MCIntegrator(4), key=0)
    f.write_text(YAML % "cylinder")
    tel = it.load_telescope(str(f), it.MCIntegrator(4), key=0)
    assert len(tel.obstruction_groups) == 1


def test_malformed_scene_file(tmp_path):
    f = tmp_path / "broken.yaml"
    f.write_text("telescope:\n  name: x\n   bad: indentation\n")
    with pytest.raises(ValueError):
        it.load_telescope(str(f), it.MCIntegrator(4), key=0)


@pytest.mark.parametrize("what", ["cylinder", "sphere", "samples", "stage"])
def test_non_finite_inputs_are_rejected_at_pack_time(what):
    groups, obst = W.davies_cotton(n_facets=7, n_samples=8, seed=1, obstructions=False)
    cam = W.hex_camera(96)
    if what == "cylinder":
        tel = Telescope(groups, group_obstructions([Cylinder([0, 0, 1], [0, 0, float("nan")], 0.1)]), [cam])
    elif what == "sphere":
        tel = Telescope(groups, group_obstructions([Sphere([0, 0, 5], float("inf"))]), [cam])
    elif what == "samples":
        g = groups[0]
        pts = g.points.clone()
        pts[0, 0, 0] = float("nan")
        tel = Telescope([g.replace(points=pts)], [], [cam])
    else:
        tel, _, _, _ = W.cassegrain(n_samples=4, n_sources=1)
        sec = [g for g in tel.mirror_groups if g.optical_stage == 1][0]
        bad = sec.replace(curvature=float("nan"))
        tel = Telescope([g if g.optical_stage == 0 else bad for g in tel.mirror_groups], [], tel.sensors)
    with pytest.raises(ValueError, match="NaN or Inf"):
        pack_scene(tel, "cpu")


def test_bad_sensor_index_raises_index_error():
    tel, src, val, st = W.plain_forward(n_samples=4, n_sources=1)
    with pytest.raises(IndexError):
        tel.sensors[3]
    assert math.isfinite(float(tel.mirror_groups[0].points.sum()))
