"""Telescope configuration loader (io/yaml_loader.py of the reference)."""
from __future__ import annotations

import torch

from ..core.apertures import DiskAperture, PolygonAperture
from ..core.obstructions import Box, Cylinder, OrientedBox, Sphere, Triangle, group_obstructions
from ..core.surfaces import AsphericSurface
from ..sensors import HexagonalSensor, SquareSensor
from ..telescope.mirrors import Mirror, group_mirrors
from ..telescope.telescope import Telescope
from ..utils import keys as _keys
from . import yamlmini


def load_telescope(filename, integrator, key=None) -> Telescope:
    """io/yaml_loader.py:29-49."""
    key = _keys.as_key(key)
    with open(filename, "r") as f:
        config = yamlmini.safe_load(f)
    return build_telescope(config, integrator, key)


def build_telescope(config, integrator, key) -> Telescope:
    """io/yaml_loader.py:52-92: only stage-0 groups are sampled."""
    key = _keys.as_key(key)
    name = (config.get("telescope") or {}).get("name", "telescope")
    templates = config.get("mirror_templates") or {}
    mirrors = [_parse_mirror(m, templates) for m in (config.get("mirrors") or [])]
    groups = []
    for g in group_mirrors(mirrors):
        if g.optical_stage == 0:
            key, sub = _keys.split(key, 2)
            groups.append(integrator.sample_group(g, sub))
        else:
            groups.append(g)
    obst = group_obstructions([_parse_obstruction(o) for o in (config.get("obstructions") or [])])
    sensors = [_parse_sensor(s) for s in (config.get("sensors") or [])]
    return Telescope(mirror_groups=groups, obstruction_groups=obst, sensors=sensors, name=name)


def _parse_mirror(m, templates) -> Mirror:
    """io/yaml_loader.py:95-112."""
    return Mirror(position=m["position"], rotation=m["orientation"],
                  surface=AsphericSurface.from_template(templates[m["template"]]),
                  aperture=_parse_aperture(m["aperture"]), optical_stage=m.get("stage", 0),
                  offset=m.get("offset", [0.0, 0.0]))


def _parse_aperture(cfg):
    """io/yaml_loader.py:115-124."""
    if cfg["type"] == "circular":
        return DiskAperture(cfg["radius"])
    if cfg["type"] == "polygon":
        return PolygonAperture(cfg["vertices"])
    raise ValueError(f"Unknown aperture type: {cfg['type']}")


def _parse_obstruction(cfg):
    """io/yaml_loader.py:127-146."""
    t = cfg["type"]
    if t == "cylinder":
        return Cylinder(cfg["p1"], cfg["p2"], cfg["r"])
    if t == "box":
        return Box(cfg["p1"], cfg["p2"])
    if t == "sphere":
        return Sphere(cfg["center"], cfg["r"])
    if t == "oriented_box":
        return OrientedBox(cfg["center"], cfg["half_extents"], cfg["rotation"])
    if t == "triangle":
        return Triangle(cfg["v0"], cfg["v1"], cfg["v2"])
    raise ValueError(f"Unknown obstruction type: {t}")


def _parse_sensor(cfg):
    """io/yaml_loader.py:149-171."""
    t = cfg["type"]
    ew = cfg.get("edge_width", 0.0)
    if t == "square":
        return SquareSensor(position=cfg["position"], rotation=cfg["orientation"], width=cfg["width"],
                            height=cfg["height"], bounds=tuple(cfg["bounds"]), edge_width=ew)
    if t == "hexagonal":
        centers = torch.tensor([cfg["centers_x"], cfg["centers_y"]], dtype=torch.float32).T
        return HexagonalSensor(position=cfg["position"], rotation=cfg["orientation"], hex_centers=centers,
                               edge_width=ew)
    raise ValueError(f"Unknown sensor type: {t}")
