"""PML and rigid boundaries (boundaries/_boundaries.py:75-417 of
rjwalters/strata-fdtd).

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
        """_boundaries.py:166-226 (uniform grids)."""
        self._solver = solver
        nx, ny, nz = solver.shape
        grid = solver.grid
        if self._max_sigma is None:
            R_target = 1e-6
            d = self.depth * grid.min_spacing
            self._max_sigma = -(self.order + 1) * solver.c * np.log(R_target) / (2 * d)
        self._sigma_x = self._create_profile(nx) if "x" in self.axes else None
        self._sigma_y = self._create_profile(ny) if "y" in self.axes else None
        self._sigma_z = self._create_profile(nz) if "z" in self.axes else None
        self._initialized = True

    def _create_profile(self, n: int) -> np.ndarray:
        """_boundaries.py:228-255: sigma_max * dist**order, float32."""
        sigma = np.zeros(n, dtype=np.float32)
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
