"""Parametric geometry and its optimisation (geometry/parametric.py of
rjwalters/strata-fdtd): shapes with named, bounded parameters, constraints
on them, and a scipy.optimize driver whose every evaluation voxelises the
candidate on the GPU."""
from __future__ import annotations

from abc import ABC, abstractmethod
from dataclasses import dataclass, field
from typing import Callable

import numpy as np


@dataclass
class Parameter:
    """A tunable dimension with its (min, max) bounds."""

    name: str
    default: float
    bounds: tuple
    unit: str = "m"
    description: str = ""

    def validate(self, value: float) -> bool:
        return self.bounds[0] <= value <= self.bounds[1]

    def clip(self, value: float) -> float:
        return np.clip(value, self.bounds[0], self.bounds[1])


class ParametricPrimitive(ABC):
    """A shape given by parameters: ``get_parameters``, ``with_parameters``
    (a new instance) and ``to_sdf`` (the concrete shape)."""

    @abstractmethod
    def get_parameters(self) -> list: ...

    @abstractmethod
    def with_parameters(self, **kwargs) -> "ParametricPrimitive": ...

    @abstractmethod
    def to_sdf(self): ...

    def to_dict(self) -> dict:
        return {p.name: getattr(self, p.name) for p in self.get_parameters()}

    @classmethod
    def from_dict(cls, params: dict) -> "ParametricPrimitive":
        return cls(**params)

    def voxelize(self, grid) -> np.ndarray:
        return self.to_sdf().voxelize(grid)


@dataclass
class ParametricHorn(ParametricPrimitive):
    """A horn along ``axis_direction`` (normalised) from ``axis_start``,
    tuned by its throat and mouth radii and its length."""

    throat_radius: float = 0.02
    mouth_radius: float = 0.06
    length: float = 0.15
    profile: str = "exponential"
    axis_start: np.ndarray = field(default_factory=lambda: np.array([0.0, 0.0, 0.0]))
    axis_direction: np.ndarray = field(default_factory=lambda: np.array([0.0, 0.0, 1.0]))

    def __post_init__(self):
        self.axis_start = np.asarray(self.axis_start, dtype=np.float64)
        self.axis_direction = np.asarray(self.axis_direction, dtype=np.float64)
        n = np.linalg.norm(self.axis_direction)
        if n > 0:
            self.axis_direction = self.axis_direction / n

    def get_parameters(self) -> list:
        return [Parameter("throat_radius", self.throat_radius, (0.005, 0.05), "m", "Throat radius"),
                Parameter("mouth_radius", self.mouth_radius, (0.02, 0.15), "m", "Mouth radius"),
                Parameter("length", self.length, (0.05, 0.5), "m", "Horn length")]

    def with_parameters(self, **kwargs) -> "ParametricHorn":
        params = dict(throat_radius=self.throat_radius, mouth_radius=self.mouth_radius,
                      length=self.length, profile=self.profile,
                      axis_start=self.axis_start.copy(),
                      axis_direction=self.axis_direction.copy())
        params.update(kwargs)
        return ParametricHorn(**params)

    def to_sdf(self):
        from .sdf import Horn

        return Horn(throat_position=tuple(self.axis_start),
                    mouth_position=tuple(self.axis_start + self.axis_direction * self.length),
                    throat_radius=self.throat_radius, mouth_radius=self.mouth_radius,
                    profile=self.profile)


@dataclass
class GeometricConstraint:
    """``expression(params)`` is the violation (> 0) or <= 0 when met."""

    name: str
    expression: Callable
    description: str = ""

    def evaluate(self, params: dict) -> float:
        return max(0, self.expression(params))


class ConstraintSet:
    """A list of constraints, with helpers for bounds and ratios."""

    def __init__(self):
        self.constraints: list = []

    def add(self, name: str, expression: Callable, description: str = ""):
        self.constraints.append(GeometricConstraint(name, expression, description))

    def add_min_value(self, param_name: str, min_value: float):
        self.add(f"min_{param_name}", lambda p: min_value - p.get(param_name, float("inf")),
                 f"{param_name} must be >= {min_value}")

    def add_max_value(self, param_name: str, max_value: float):
        self.add(f"max_{param_name}", lambda p: p.get(param_name, -float("inf")) - max_value,
                 f"{param_name} must be <= {max_value}")

    def add_ratio_constraint(self, param_a: str, param_b: str, min_ratio: float):
        """param_b >= min_ratio * param_a (met trivially when param_a is 0)."""
        def check(p):
            a, b = p.get(param_a, 0), p.get(param_b, 0)
            return 0 if a == 0 else a * min_ratio - b

        self.add(f"{param_b}_over_{param_a}", check, f"{param_b}/{param_a} must be >= {min_ratio}")

    def evaluate_all(self, params: dict) -> dict:
        return {c.name: c.evaluate(params) for c in self.constraints}

    def is_feasible(self, params: dict) -> bool:
        return all(v <= 1e-10 for v in self.evaluate_all(params).values())

    def total_violation(self, params: dict) -> float:
        return sum(self.evaluate_all(params).values())


class GeometryOptimizer:
    """Minimises ``objective_fn(mask)`` over a parametric shape's
    parameters; infeasible points cost 1e6 (1 + violation), shapes that fail
    to build or voxelise 1e9."""

    def __init__(self, geometry: ParametricPrimitive, grid, constraints=None):
        self.geometry, self.grid = geometry, grid
        self.constraints = constraints or ConstraintSet()
        self._param_names = [p.name for p in geometry.get_parameters()]
        self._param_bounds = [p.bounds for p in geometry.get_parameters()]

    def objective(self, params_vector, objective_fn) -> float:
        params = dict(zip(self._param_names, params_vector))
        violation = self.constraints.total_violation(params)
        if violation > 1e-10:
            return 1e6 * (1 + violation)
        try:
            mask = self.geometry.with_parameters(**params).voxelize(self.grid)
        except Exception:
            return 1e9
        return objective_fn(mask)

    def optimize(self, objective_fn, method: str = "Nelder-Mead", **scipy_options) -> dict:
        from scipy.optimize import minimize

        x0 = np.array([p.default for p in self.geometry.get_parameters()])
        res = minimize(lambda x: self.objective(x, objective_fn), x0, method=method,
                       bounds=self._param_bounds, **scipy_options)
        best = dict(zip(self._param_names, res.x))
        return {"parameters": best, "objective": res.fun, "success": res.success,
                "geometry": self.geometry.with_parameters(**best), "message": res.message,
                "nfev": res.nfev}
