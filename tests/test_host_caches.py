"""Host-side caches of the render path are invalidated by every change
that must reach the kernels: packed sensor descriptors (pose tensors
replaced by the editors or modified in place, scalar settings), stage
grouping (edited mirror-group lists) and packed scenes (sample arrays
modified in place). CPU only: descriptors are host structs."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from iactrace_gb300 import workloads as W
from iactrace_gb300.core.scene import stages_of
from iactrace_gb300.sensors import SquareSensor


def _pos(desc):
    return tuple(desc.pos[i] for i in range(3))


def test_sensor_descriptor_follows_pose_and_settings():
    cam = SquareSensor([0.0, 0.0, 15.0], [0.0, 0.0, 0.0], 32, 30, (-0.672, 0.672, -0.63, 0.63))
    d1, _ = cam.pack("cpu")
    d2, _ = cam.pack("cpu")
    assert d1 is d2  # cached
    cam.position[2] += 0.5  # in place: new version
    d3, _ = cam.pack("cpu")
    assert _pos(d3)[2] == np.float32(15.5)
    cam.position = torch.tensor([0.1, 0.0, 15.0])  # replaced
    d4, _ = cam.pack("cpu")
    assert abs(_pos(d4)[0] - 0.1) < 1e-7
    cam.edge_width = 0.004  # scalar setting
    d5, _ = cam.pack("cpu")
    assert abs(d5.edge_width - 0.004) < 1e-9
    assert d5 is not d4


def test_editor_moves_reach_the_descriptor():
    tel, src, val, st = W.plain_forward(n_samples=8, n_sources=2)
    d0, _ = tel.sensors[0].pack("cpu")
    tel2 = tel.set_sensor_position(0, [0.0, 0.0, 14.0])
    d1, _ = tel2.sensors[0].pack("cpu")
    assert _pos(d1)[2] == np.float32(14.0)
    assert _pos(d0)[2] == np.float32(15.0)  # the original telescope is unchanged


def test_stage_grouping_follows_the_group_list():
    tel, src, val, st = W.cassegrain(n_samples=4, n_sources=2)
    s1 = stages_of(tel)
    assert stages_of(tel) is s1 and sorted(s1) == [0, 1]
    tel.mirror_groups = tel.mirror_groups[:1]  # edited list
    assert sorted(stages_of(tel)) == [0]


def test_packed_scene_follows_in_place_sample_changes():
    from iactrace_gb300.core.scene import pack_scene
    tel, src, val, st = W.plain_forward(n_samples=8, n_sources=2)
    a = pack_scene(tel, "cpu")
    assert pack_scene(tel, "cpu") is a
    g = tel.mirror_groups[0]
    with torch.no_grad():
        g.points[0, 0, 2] += 0.25  # in place
    b = pack_scene(tel, "cpu")
    assert b is not a
    assert float(b.points[0, 0, 2]) == float(g.points[0, 0, 2])


def test_packed_scene_rejects_non_finite_samples():
    from iactrace_gb300.core.scene import pack_scene
    tel, src, val, st = W.plain_forward(n_samples=8, n_sources=2)
    g = tel.mirror_groups[0]
    with torch.no_grad():
        g.normals[1, 2, 0] = float("nan")
    try:
        pack_scene(tel, "cpu")
    except ValueError as e:
        assert "NaN" in str(e)
    else:
        raise AssertionError("a NaN normal was packed")


def test_fast_launch_key_follows_every_change():
    """The key that lets repeated renders skip packing changes with every
    edit that must reach the kernels, and is None on the autograd path."""
    from iactrace_gb300.core.render import _state_key
    from iactrace_gb300.core import Cylinder, group_obstructions
    tel, src, val, st = W.plain_forward(n_samples=8, n_sources=2)
    cam = tel.sensors[0]
    k0 = _state_key(tel, cam)
    assert k0 is not None and _state_key(tel, cam) == k0
    g = tel.mirror_groups[0]
    with torch.no_grad():
        g.rotations[3, 0] += 0.01  # facet transform in place
    k1 = _state_key(tel, cam)
    assert k1 != k0
    with torch.no_grad():
        g.weights[0, 0] *= 2.0  # sample array in place
    k2 = _state_key(tel, cam)
    assert k2 != k1
    g.perturbation_scale = g.perturbation_scale + 1e-6  # field replaced
    k3 = _state_key(tel, cam)
    assert k3 != k2
    cam.position[2] += 0.1  # sensor pose in place
    k4 = _state_key(tel, cam)
    assert k4 != k3
    cam.edge_width = 0.003  # sensor setting
    k5 = _state_key(tel, cam)
    assert k5 != k4
    tel.obstruction_groups = list(tel.obstruction_groups) + group_obstructions([Cylinder([0, 0, 1], [0, 0, 2], 0.1)])
    k6 = _state_key(tel, cam)
    assert k6 != k5
    tel2 = tel.set_mirror_rotations(0, g.rotations.clone().requires_grad_(True))
    assert _state_key(tel2, tel2.sensors[0]) is None


def test_fast_launch_validation_sees_what_the_key_sees():
    """The per-call check of the fast forward path (object identities plus
    the version counters of the tensor fields) changes whenever _state_key
    does, for each kind of edit."""
    from iactrace_gb300.core.render import _object_ids, _state_key, _tensor_fields
    from iactrace_gb300.core import Cylinder, group_obstructions
    tel, src, val, st = W.plain_forward(n_samples=8, n_sources=2)
    cam = tel.sensors[0]

    def check():
        return _object_ids(tel, cam), tuple(t._version for t in _tensor_fields(tel, cam))

    c0, k0 = check(), _state_key(tel, cam)
    assert check() == c0
    g = tel.mirror_groups[0]
    def rotate():
        with torch.no_grad():
            g.rotations[3, 0] += 0.01  # facet transform in place

    edits = [
        rotate,
        lambda: setattr(g, "perturbation_scale", g.perturbation_scale + 1e-6),
        lambda: cam.position.__setitem__(2, cam.position[2] + 0.1),
        lambda: setattr(cam, "edge_width", 0.003),
        lambda: setattr(tel, "obstruction_groups",
                        list(tel.obstruction_groups) + group_obstructions([Cylinder([0, 0, 1], [0, 0, 2], 0.1)])),
    ]
    for edit in edits:
        edit()
        c1, k1 = check(), _state_key(tel, cam)
        assert k1 != k0 and c1 != c0
        c0, k0 = c1, k1
