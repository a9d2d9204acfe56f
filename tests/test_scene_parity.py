"""Host-side scene construction against the reference's own (fixtures
written by tests/golden/make_scene_golden.py from GerritRo/iactrace on the
numpy stand-in, float32):

* load_telescope of the HESS CT3 and CT5 configurations (io/yaml_loader.py:
  29-171): mirror-group partition and every deterministic field of the
  groups (telescope/mirrors.py:232-313), obstruction groups and tables
  (core/obstructions.py:258-277), sensors with their pixel geometry, hexagon
  grid constants and lookup tables: equal bit for bit;
* the editors of telescope/operations.py:87-229 and :360-373 on the loaded
  CT3: equal bit for bit, with the reference's own unit-normal draws fed to
  the random editors (their streams differ: threefry vs Philox), so what is
  compared is the mapping from draws to parameters (arcsec to degrees, which
  Euler angle, which coordinate).

CPU only; the YAML files come from a checkout of the reference.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest
import torch

import iactrace_gb300 as it
from iactrace_gb300.telescope import operations as ops

HERE = os.path.dirname(os.path.abspath(__file__))
OBST_FIELDS = {"CylinderGroup": ("p1", "p2", "r"), "BoxGroup": ("p1", "p2"), "SphereGroup": ("centers", "radii"),
               "OrientedBoxGroup": ("centers", "half_extents", "rotations"), "TriangleGroup": ("v0", "v1", "v2")}


def _fixture(name):
    p = os.path.join(HERE, "golden", f"{name}.npz")
    if not os.path.exists(p):
        pytest.skip("fixture not generated")
    return dict(np.load(p, allow_pickle=False))


def _np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


def _load(reference_checkout, name):
    path = os.path.join(reference_checkout, "configs", "HESS", f"{name}.yaml")
    return it.load_telescope(path, it.MCIntegrator(2), 0)


def _same(a, b, what):
    a, b = _np(a), _np(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if a.dtype.kind == "f" or b.dtype.kind == "f":
        assert a.dtype == np.float32 and b.dtype == np.float32, f"{what}: dtypes {a.dtype} / {b.dtype}"
    assert np.array_equal(a, b), f"{what}: {int((a != b).sum())} entries differ, max {np.abs(a - b).max():.3g}"


@pytest.mark.parametrize("name", ["CT3", "CT5"])
def test_loader_matches_reference(reference_checkout, name):
    fx = _fixture(f"loader_{name}")
    meta = json.loads(str(fx["meta"]))
    tel = _load(reference_checkout, name)
    assert tel.name == meta["name"]
    assert len(tel.mirror_groups) == len(meta["groups"])
    for i, (g, d) in enumerate(zip(tel.mirror_groups, meta["groups"])):
        assert type(g).__name__ == d["class"] and g.optical_stage == d["stage"] and len(g) == d["n"], i
        assert np.float32(float(g.curvature)) == np.float32(d["curvature"])
        assert np.float32(float(g.conic)) == np.float32(d["conic"])
        for k in ("positions", "rotations", "offsets", "aspheric", "perturbation_scale"):
            _same(getattr(g, k), fx[f"g{i}_{k}"], f"group {i} {k}")
        k = "radii" if f"g{i}_radii" in fx else "vertices"
        _same(getattr(g, k), fx[f"g{i}_{k}"], f"group {i} {k}")
    groups = tel.obstruction_groups or []
    assert [type(g).__name__ for g in groups] == meta["obstructions"]
    for i, g in enumerate(groups):
        for k in OBST_FIELDS[type(g).__name__]:
            _same(getattr(g, k), fx[f"o{i}_{k}"], f"obstruction group {i} {k}")
    assert len(tel.sensors) == len(meta["sensors"])
    for i, (s, d) in enumerate(zip(tel.sensors, meta["sensors"])):
        assert type(s).__name__ == d["class"], i
        _same(s.position, fx[f"s{i}_position"], f"sensor {i} position")
        _same(s.rotation, fx[f"s{i}_rotation"], f"sensor {i} rotation")
        assert float(s.edge_width) == d["edge_width"]
        if "Square" in d["class"]:
            assert (s.width, s.height) == (d["width"], d["height"])
            assert (s.x0, s.y0, s.dx, s.dy) == (d["x0"], d["y0"], d["dx"], d["dy"])
        else:
            assert (s.hex_size, s.hex_inradius, s.grid_rotation) == (d["hex_size"], d["hex_inradius"],
                                                                     d["grid_rotation"])
            assert list(s.grid_offset) == d["grid_offset"]
            assert (s.q_min, s.r_min, s.n_pixels) == (d["q_min"], d["r_min"], d["n_pixels"])
            _same(s.hex_centers, fx[f"s{i}_hex_centers"], f"sensor {i} centres")
            assert np.array_equal(_np(s.lookup_table), fx[f"s{i}_lookup_table"])


def test_editors_match_reference(reference_checkout, monkeypatch):
    fx = _fixture("editors_CT3")
    tel = _load(reference_checkout, "CT3")
    g0 = tel.mirror_groups[0]
    _same(g0.rotations, fx["rotations0"], "rotations")
    _same(g0.positions, fx["positions0"], "positions")
    w0 = fx["weights0"]
    # weights come from the (differently seeded) sampler: edit the reference's
    # own weights so that the scaling itself is compared
    tel = ops._with_group(tel, 0, g0.replace(weights=torch.from_numpy(w0)))
    assert np.float32(ops.apply_roughness(tel, 24.0).mirror_groups[0].perturbation_scale[0]) == \
        fx["roughness_scale"][0, 0]
    _same(ops.apply_roughness(tel, 24.0).mirror_groups[0].perturbation_scale.float(), fx["roughness_scale"][0],
          "apply_roughness")
    _same(ops.apply_roughness_to_group(tel, 0, 12.0).mirror_groups[0].perturbation_scale.float(),
          fx["roughness_group_scale"], "apply_roughness_to_group")
    _same(ops.scale_mirror_weights(tel, 0, 0.8).mirror_groups[0].weights, fx["weights_scalar"],
          "scale_mirror_weights (scalar)")
    _same(ops.scale_mirror_weights(tel, 0, torch.from_numpy(fx["weight_factors"])).mirror_groups[0].weights,
          fx["weights_per_mirror"], "scale_mirror_weights (per mirror)")
    _same(ops.set_mirror_rotations(tel, 0, _np(g0.rotations) + np.float32(0.01)).mirror_groups[0].rotations,
          fx["set_rotations"], "set_mirror_rotations")
    _same(ops.set_mirror_positions(tel, 0, _np(g0.positions) * np.float32(1.001)).mirror_groups[0].positions,
          fx["set_positions"], "set_mirror_positions")
    _same(ops.focus(tel, 0.01, 0).sensors[0].position, fx["focus_position"], "focus")

    draws = []
    real_randn = torch.randn

    def fed_randn(*shape, generator=None, **kw):
        return torch.from_numpy(draws.pop(0)) if draws else real_randn(*shape, generator=generator, **kw)

    monkeypatch.setattr(torch, "randn", fed_randn)
    draws[:] = [fx["misalign_z_h"], fx["misalign_z_v"]]
    out = ops.apply_misalignment_to_group(tel, 0, 20.0, 35.0, 5).mirror_groups[0].rotations
    assert not draws
    _same(out, fx["misalign_rotations"], "apply_misalignment_to_group")
    draws[:] = [fx["displace_z"]]
    out = ops.apply_displacement_to_group(tel, 0, 0.003, 6).mirror_groups[0].positions
    assert not draws
    _same(out, fx["displace_positions"], "apply_displacement_to_group")
