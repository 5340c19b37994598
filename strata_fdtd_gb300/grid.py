"""Uniform grid (core/grid.py:51-146 of rjwalters/strata-fdtd).

Cell centres are ``np.arange(n) * resolution + resolution / 2``; the SDF
voxeliser evaluates geometry at exactly these FP64 coordinates.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class UniformGrid:
    shape: tuple[int, int, int]
    resolution: float
    _x: np.ndarray = field(init=False, repr=False)
    _y: np.ndarray = field(init=False, repr=False)
    _z: np.ndarray = field(init=False, repr=False)

    def __post_init__(self):
        self.shape = tuple(int(n) for n in self.shape)
        if len(self.shape) != 3 or min(self.shape) < 1:
            raise ValueError(f"shape must be three positive integers, got {self.shape}")
        if self.resolution <= 0:
            raise ValueError("resolution must be positive")
        r = self.resolution
        self._x = np.arange(self.shape[0]) * r + r / 2
        self._y = np.arange(self.shape[1]) * r + r / 2
        self._z = np.arange(self.shape[2]) * r + r / 2

    @property
    def x_coords(self):
        return self._x

    @property
    def y_coords(self):
        return self._y

    @property
    def z_coords(self):
        return self._z

    @property
    def dx(self):
        return np.full(self.shape[0], self.resolution)

    @property
    def dy(self):
        return np.full(self.shape[1], self.resolution)

    @property
    def dz(self):
        return np.full(self.shape[2], self.resolution)

    @property
    def min_spacing(self) -> float:
        return self.resolution

    @property
    def max_spacing(self) -> float:
        return self.resolution

    @property
    def is_uniform(self) -> bool:
        return True

    @property
    def num_cells(self) -> int:
        return int(np.prod(self.shape))

    def physical_extent(self):
        return tuple(n * self.resolution for n in self.shape)
