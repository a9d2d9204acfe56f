"""Functional telescope editors (telescope/operations.py of the reference).

Each returns a new Telescope; inputs are never modified in place.
"""
from __future__ import annotations

import copy
import math

import torch

from ..utils import keys as _keys


def _replace(tel, **fields):
    t = copy.copy(tel)
    t.__dict__.pop("_packed", None)
    for k, v in fields.items():
        setattr(t, k, v)
    return t


def _with_group(tel, idx, group):
    groups = list(tel.mirror_groups)
    groups[idx] = group
    return _replace(tel, mirror_groups=groups)


def resample_mirrors(telescope, integrator, key):
    """operations.py:25-40: resample every group."""
    ks = _keys.split(key, len(telescope.mirror_groups))
    return _replace(telescope, mirror_groups=[integrator.sample_group(g, k)
                                              for g, k in zip(telescope.mirror_groups, ks)])


def set_mirror_positions(telescope, group_idx, positions):
    """operations.py:43-62."""
    g = telescope.mirror_groups[group_idx]
    return _with_group(telescope, group_idx, g.replace(positions=torch.as_tensor(positions, dtype=torch.float32)))


def set_mirror_rotations(telescope, group_idx, rotations):
    """operations.py:65-84 (Euler degrees)."""
    g = telescope.mirror_groups[group_idx]
    return _with_group(telescope, group_idx, g.replace(rotations=torch.as_tensor(rotations, dtype=torch.float32)))


def scale_mirror_weights(telescope, group_idx, scale_factors):
    """operations.py:87-115: weights (N,M,1) * scale (N,)."""
    g = telescope.mirror_groups[group_idx]
    s = torch.as_tensor(scale_factors, dtype=torch.float32)
    if s.ndim == 0:
        s = torch.full((len(g),), float(s))
    return _with_group(telescope, group_idx, g.replace(weights=g.weights * s[:, None, None]))


def apply_roughness(telescope, roughness):
    """operations.py:118-135: roughness in arcsec -> perturbation_scale in rad."""
    sigma = roughness * math.pi / (180.0 * 3600.0)
    return _replace(telescope, mirror_groups=[g.replace(perturbation_scale=torch.full((len(g),), sigma))
                                              for g in telescope.mirror_groups])


def apply_roughness_to_group(telescope, group_idx, roughness):
    """operations.py:138-158."""
    sigma = roughness * math.pi / (180.0 * 3600.0)
    g = telescope.mirror_groups[group_idx]
    return _with_group(telescope, group_idx, g.replace(perturbation_scale=torch.full((len(g),), sigma)))


def apply_misalignment_to_group(telescope, group_idx, sigma_h, sigma_v, key):
    """operations.py:161-198: Gaussian tip/tilt errors, sigmas in arcsec."""
    g = telescope.mirror_groups[group_idx]
    k1, k2 = _keys.split(key, 2)
    dh = torch.randn(len(g), generator=_keys.generator(k1)) * (sigma_h / 3600.0)
    dv = torch.randn(len(g), generator=_keys.generator(k2)) * (sigma_v / 3600.0)
    rot = g.rotations.clone()
    rot[:, 0] += dh
    rot[:, 1] += dv
    return _with_group(telescope, group_idx, g.replace(rotations=rot))


def apply_displacement_to_group(telescope, group_idx, sigma_z, key):
    """operations.py:201-229: Gaussian z displacement of facet positions."""
    g = telescope.mirror_groups[group_idx]
    pos = g.positions.clone()
    pos[:, 2] += torch.randn(len(g), generator=_keys.generator(key)) * sigma_z
    return _with_group(telescope, group_idx, g.replace(positions=pos))


def get_mirrors_by_stage(telescope, stage):
    """operations.py:232-244."""
    return [i for i, g in enumerate(telescope.mirror_groups) if g.optical_stage == stage]


def get_mirror_count(telescope):
    """operations.py:247-259."""
    return sum(len(g) for g in telescope.mirror_groups)


def add_sensor(telescope, sensor):
    """operations.py:262-273."""
    return _replace(telescope, sensors=list(telescope.sensors) + [sensor])


def replace_sensor(telescope, sensor, idx=0):
    """operations.py:276-296."""
    if idx < 0 or idx >= len(telescope.sensors):
        raise IndexError(f"Sensor index {idx} out of range (0-{len(telescope.sensors) - 1})")
    s = list(telescope.sensors)
    s[idx] = sensor
    return _replace(telescope, sensors=s)


def remove_sensor(telescope, idx=0):
    """operations.py:299-319."""
    if idx < 0 or idx >= len(telescope.sensors):
        raise IndexError(f"Sensor index {idx} out of range (0-{len(telescope.sensors) - 1})")
    return _replace(telescope, sensors=[s for i, s in enumerate(telescope.sensors) if i != idx])


def _sensor_field(telescope, idx, **fields):
    s = copy.copy(telescope.sensors[idx])
    for k, v in fields.items():
        setattr(s, k, v)
    return replace_sensor(telescope, s, idx)


def set_sensor_position(telescope, idx, position):
    """operations.py:320-337."""
    return _sensor_field(telescope, idx, position=torch.as_tensor(position, dtype=torch.float32).reshape(3))


def set_sensor_rotation(telescope, idx, rotation):
    """operations.py:340-357."""
    return _sensor_field(telescope, idx, rotation=torch.as_tensor(rotation, dtype=torch.float32).reshape(3))


def focus(telescope, delta_z, sensor_idx=0):
    """operations.py:360-373: move the sensor along z."""
    pos = telescope.sensors[sensor_idx].position.clone()
    pos[2] += delta_z
    return set_sensor_position(telescope, sensor_idx, pos)


def get_sensor_count(telescope):
    return len(telescope.sensors)


def add_obstruction(telescope, obstruction):
    """operations.py:391-405."""
    return _replace(telescope, obstruction_groups=list(telescope.obstruction_groups or []) + [obstruction])


def remove_obstruction(telescope, group_idx):
    """operations.py:408-431."""
    if not telescope.obstruction_groups:
        raise IndexError("No obstruction groups to remove")
    if group_idx < 0 or group_idx >= len(telescope.obstruction_groups):
        raise IndexError(f"Obstruction group index {group_idx} out of range "
                         f"(0-{len(telescope.obstruction_groups) - 1})")
    return _replace(telescope, obstruction_groups=[g for i, g in enumerate(telescope.obstruction_groups)
                                                   if i != group_idx])


def clear_obstructions(telescope):
    """operations.py:434-444."""
    return _replace(telescope, obstruction_groups=[])


def get_obstruction_count(telescope):
    """operations.py:447-457."""
    return sum(len(g) for g in (telescope.obstruction_groups or []))


def clone(telescope):
    """operations.py:463-472: deep copy."""
    t = copy.deepcopy(telescope)
    t.__dict__.pop("_packed", None)
    return t


def get_info(telescope):
    """operations.py:475-541."""
    from ..sensors import HexagonalSensor, SquareSensor
    from .mirrors import AsphericDiskMirrorGroup, AsphericPolygonMirrorGroup
    types = ["disk" if isinstance(g, AsphericDiskMirrorGroup) else
             "polygon" if isinstance(g, AsphericPolygonMirrorGroup) else "unknown" for g in telescope.mirror_groups]
    stypes = ["hexagonal" if isinstance(s, HexagonalSensor) else "square" if isinstance(s, SquareSensor)
              else type(s).__name__ for s in telescope.sensors]
    if telescope.mirror_groups:
        allp = torch.cat([g.positions for g in telescope.mirror_groups])
        bmin, bmax = allp.min(0).values, allp.max(0).values
    else:
        bmin = bmax = torch.zeros(3)
    return {
        "name": telescope.name,
        "n_mirror_groups": len(telescope.mirror_groups),
        "n_mirrors": get_mirror_count(telescope),
        "optical_stages": sorted({g.optical_stage for g in telescope.mirror_groups}),
        "mirror_types": types,
        "n_sensors": len(telescope.sensors),
        "sensor_types": stypes,
        "n_obstruction_groups": len(telescope.obstruction_groups or []),
        "n_obstructions": get_obstruction_count(telescope),
        "bbox_min": bmin,
        "bbox_max": bmax,
    }
