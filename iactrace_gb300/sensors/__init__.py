from .hexagonal import DifferentiableHexagonalSensor, HexagonalSensor
from .square import DifferentiableSquareSensor, SquareSensor

__all__ = ["SquareSensor", "HexagonalSensor", "DifferentiableSquareSensor", "DifferentiableHexagonalSensor"]
