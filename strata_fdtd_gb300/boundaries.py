"""PML, rigid, Mur ABC and radiation-impedance boundaries
(boundaries/_boundaries.py:75-793 of rjwalters/strata-fdtd).

The reference PML is a multiplicative decay exp(-sigma*dt) applied to the
velocity and pressure after each step; its CPML auxiliary arrays are
allocated but never used.  Here the sigma profile is computed on the host in
the reference's arithmetic and handed to the GPU plan, which forms the decay
factors in float exactly as initialize_pml (pml.cpp:13-45) does and applies
them inside the fused step kernel.
"""
from __future__ import annotations

from typing import Literal

import numpy as np


class RigidBoundary:
    """Perfect reflection; built into the geometry handling (no-op)."""

    def initialize(self, solver) -> None:
        pass

    def reset(self) -> None:
        pass


class PML:
    """Perfectly matched layer: polynomial sigma profile of ``depth`` cells
    on both ends of each selected axis (``axis`` 'all', 'x', 'y', 'z' or a
    tuple), target reflection 1e-6 unless ``max_sigma`` is given."""

    def __init__(self, depth: int = 10,
                 axis: Literal["all", "x", "y", "z"] | tuple[str, ...] = "all",
                 max_sigma: float | None = None, order: int = 3):
        self.depth = depth
        self.order = order
        if axis == "all":
            self.axes = ("x", "y", "z")
        elif isinstance(axis, str):
            self.axes = (axis,)
        else:
            self.axes = tuple(axis)
        self._max_sigma = max_sigma
        self._initialized = False
        self._sigma_x = self._sigma_y = self._sigma_z = None
        self._solver = None

    def initialize(self, solver) -> None:
        """_boundaries.py:166-226: index profiles on uniform grids, physical
        distance profiles on nonuniform ones."""
        self._solver = solver
        nx, ny, nz = solver.shape
        grid = solver.grid
        if self._max_sigma is None:
            R_target = 1e-6
            d = self.depth * grid.min_spacing
            self._max_sigma = -(self.order + 1) * solver.c * np.log(R_target) / (2 * d)
        if grid.is_uniform:
            self._sigma_x = self._create_profile(nx) if "x" in self.axes else None
            self._sigma_y = self._create_profile(ny) if "y" in self.axes else None
            self._sigma_z = self._create_profile(nz) if "z" in self.axes else None
        else:
            self._sigma_x = (self._create_profile_nonuniform(grid.x_coords, grid.dx)
                             if "x" in self.axes else None)
            self._sigma_y = (self._create_profile_nonuniform(grid.y_coords, grid.dy)
                             if "y" in self.axes else None)
            self._sigma_z = (self._create_profile_nonuniform(grid.z_coords, grid.dz)
                             if "z" in self.axes else None)
        self._initialized = True

    def _create_profile_nonuniform(self, coords, cell_spacing) -> np.ndarray:
        """_boundaries.py:257-315: sigma_max * (distance from the PML
        interface / PML thickness)**order, distances in metres; a depth of
        half the axis or more falls back to a quarter of it."""
        n = len(coords)
        sigma = np.zeros(n, dtype=np.float32)
        d = self.depth
        if d >= n // 2:
            d = max(1, n // 4)
        left_thickness = float(np.sum(cell_spacing[:d]))
        right_thickness = float(np.sum(cell_spacing[-d:]))
        left_interface = coords[d] - cell_spacing[d] / 2 if d < n else coords[-1]
        right_interface = (coords[n - d - 1] + cell_spacing[n - d - 1] / 2
                           if n - d > 0 else coords[0])
        for i in range(d):
            dist = left_interface - coords[i]
            nd = min(1.0, dist / left_thickness) if left_thickness > 0 else 0.0
            sigma[i] = self._max_sigma * (nd ** self.order)
        for i in range(n - d, n):
            dist = coords[i] - right_interface
            nd = min(1.0, dist / right_thickness) if right_thickness > 0 else 0.0
            sigma[i] = self._max_sigma * (nd ** self.order)
        return sigma

    def _create_profile(self, n: int, dtype=np.float32) -> np.ndarray:
        """_boundaries.py:228-255: sigma_max * dist**order, float32 (float64
        for the differentiable solve's double and double-word forms)."""
        sigma = np.zeros(n, dtype=dtype)
        d = self.depth
        for i in range(d):
            dist = (d - i) / d
            sigma[i] = self._max_sigma * (dist ** self.order)
        for i in range(n - d, n):
            dist = (i - (n - d - 1)) / d
            sigma[i] = self._max_sigma * (dist ** self.order)
        return sigma

    @property
    def sigmas(self):
        return self._sigma_x, self._sigma_y, self._sigma_z

    def get_interior_slice(self):
        if self._solver is None:
            raise RuntimeError("PML not initialized")
        d = self.depth
        nx, ny, nz = self._solver.shape
        return (slice(d, nx - d) if "x" in self.axes else slice(None),
                slice(d, ny - d) if "y" in self.axes else slice(None),
                slice(d, nz - d) if "z" in self.axes else slice(None))

    @property
    def is_initialized(self) -> bool:
        return self._initialized

    def reset(self) -> None:
        pass


class ABCFirstOrder:
    """First-order Mur absorbing boundary on the pressure planes of the
    selected axes (_boundaries.py:420-527): after the step, for x then y then
    z, p[0] = prev0 + m (p[1] - p[0]) and prev0 = p[1], then the same at the
    high end, with m = (c dt - dx) / (c dt + dx).  m is a NumPy float64
    (dt is), so the update runs in FP64 on the float32 difference and rounds
    once into p, as NumPy does it."""

    def __init__(self, axis: Literal["all", "x", "y", "z"] | tuple[str, ...] = "all"):
        if axis == "all":
            self.axes = ("x", "y", "z")
        elif isinstance(axis, str):
            self.axes = (axis,)
        else:
            self.axes = tuple(axis)
        self._solver = None
        self._coeff = 0.0

    def initialize(self, solver) -> None:
        self._solver = solver
        self._coeff = (solver.c * solver.dt - solver.dx) / (solver.c * solver.dt + solver.dx)

    def plane_ops(self):
        """(kind, axis, side, coefficient, reflection) entries, in order."""
        return [(0, "xyz".index(a), 2, float(self._coeff), 0.0) for a in ("x", "y", "z")
                if a in self.axes]

    def apply_velocity(self, solver) -> None:
        pass

    def reset(self) -> None:
        if self._solver is not None:
            self._solver._plane_bc_dirty = True


class RadiationImpedance:
    """Partially reflecting open end of one axis (_boundaries.py:529-793):
    p_b = R p_i + (1 - R) (prev + m (p_i - p_b)), prev = p_i, with m the Mur
    coefficient (a NumPy float64) and R either the given reflection
    coefficient or, from ``pipe_radius``, |(z - 1)/(z + 1)| clamped to 0.95
    with z = (ka)^2 / 4 at k = 2 pi 1 kHz / c."""

    def __init__(self, axis: Literal["x", "y", "z"], side: Literal["low", "high"],
                 reflection_coeff: float | None = None, pipe_radius: float | None = None):
        self.axis = axis
        self.side = side
        if reflection_coeff is not None:
            if not 0.0 <= reflection_coeff <= 1.0:
                raise ValueError("reflection_coeff must be in [0, 1]")
            self._reflection_coeff = reflection_coeff
            self._frequency_dependent = False
        elif pipe_radius is not None:
            if pipe_radius <= 0:
                raise ValueError("pipe_radius must be positive")
            self._pipe_radius = pipe_radius
            self._frequency_dependent = True
            self._reflection_coeff = None
        else:
            raise ValueError("Must specify either reflection_coeff or pipe_radius")
        self._solver = None
        self._initialized = False
        self._coeff_a = 0.0
        self._coeff_b = 0.0

    def initialize(self, solver) -> None:
        self._solver = solver
        c, dt, dx = solver.c, solver.dt, solver.dx
        if not self._frequency_dependent:
            R = self._reflection_coeff
        else:
            k_char = 2 * np.pi * 1000 / c
            ka = k_char * self._pipe_radius
            z_ratio = (ka ** 2) / 4
            R = abs((z_ratio - 1) / (z_ratio + 1))
            R = min(R, 0.95)
        mur_coeff = (c * dt - dx) / (c * dt + dx)
        self._coeff_a = (1 - R) * mur_coeff
        self._coeff_b = R
        self._mur = mur_coeff
        self._initialized = True

    def plane_ops(self):
        return [(1, "xyz".index(self.axis), 0 if self.side == "low" else 1, float(self._mur),
                 float(self._coeff_b))]

    def apply_velocity(self, solver) -> None:
        pass

    def reset(self) -> None:
        if self._solver is not None:
            self._solver._plane_bc_dirty = True

    @property
    def reflection_coefficient(self) -> float:
        return self._coeff_b

    @property
    def is_initialized(self) -> bool:
        return self._initialized
