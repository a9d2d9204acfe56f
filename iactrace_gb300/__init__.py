"""iactrace_gb300: the IACTrace render path on GB300 (sm_103a).

Same public names as the reference package (GerritRo/iactrace v0.4.0,
iactrace/__init__.py): Telescope, Mirror, Integrator, MCIntegrator,
SquareSensor, HexagonalSensor, load_telescope; plotting data (no drawing) is in
iactrace_gb300.viz. Rendering runs in hand-written CUDA kernels behind a C ABI
(include/iactrace_gb300.h).
"""
from .core import (BatchRenderer, DeviceIntegrator, Integrator, MCIntegrator, RenderPlan, render, render_debug,
                   render_response_matrix)
from .io import load_telescope
from .sensors import DifferentiableHexagonalSensor, DifferentiableSquareSensor, HexagonalSensor, SquareSensor
from .telescope import Mirror, Telescope

__version__ = "0.4.0+gb300.1"

__all__ = [
    "Telescope", "Mirror", "Integrator", "MCIntegrator", "SquareSensor", "HexagonalSensor",
    "DifferentiableSquareSensor", "DifferentiableHexagonalSensor", "load_telescope",
    "render", "render_debug", "render_response_matrix", "BatchRenderer", "DeviceIntegrator", "RenderPlan",
]
