from .apertures import Aperture, DiskAperture, PolygonAperture
from .batch import BatchRenderer
from .integrators import DeviceIntegrator, Integrator, MCIntegrator
from .obstructions import (Box, BoxGroup, Cylinder, CylinderGroup, Obstruction, ObstructionGroup, OrientedBox,
                           OrientedBoxGroup, Sphere, SphereGroup, Triangle, TriangleGroup, group_obstructions)
from .plan import RenderPlan
from .reflection import compute_perturbation_delta, reflect
from .render import render, render_debug, render_response_matrix
from .surfaces import AsphericSurface
from .transforms import euler_to_matrix, look_at_euler, look_at_rotation

__all__ = [
    "AsphericSurface", "Aperture", "DiskAperture", "PolygonAperture", "Integrator", "MCIntegrator", "DeviceIntegrator",
    "compute_perturbation_delta", "reflect", "euler_to_matrix", "look_at_rotation", "look_at_euler",
    "render", "render_debug", "render_response_matrix", "BatchRenderer", "RenderPlan",
    "Obstruction", "ObstructionGroup", "Cylinder", "CylinderGroup", "Box", "BoxGroup", "Sphere", "SphereGroup",
    "OrientedBox", "OrientedBoxGroup", "Triangle", "TriangleGroup", "group_obstructions",
]
