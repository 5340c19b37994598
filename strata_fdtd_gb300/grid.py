"""Uniform and nonuniform grids (core/grid.py:51-532 of rjwalters/strata-fdtd).

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


class NonuniformGrid:
    """Variable spacing from cell-centre coordinates per axis (core/grid.py:
    148-532 of rjwalters/strata-fdtd): spacing[i] = (x[i+1] - x[i-1]) / 2
    inside, the neighbour distance at both ends; the stencil's face
    spacings are the centre distances.  Same constructors and properties as
    the reference, with its FP64 arithmetic (the spacing arrays handed to the
    kernels are rounded to float32 as the reference rounds them)."""

    def __init__(self, x_coords, y_coords, z_coords):
        self._x_coords = np.asarray(x_coords, dtype=np.float64).ravel()
        self._y_coords = np.asarray(y_coords, dtype=np.float64).ravel()
        self._z_coords = np.asarray(z_coords, dtype=np.float64).ravel()
        for name, c in (("x", self._x_coords), ("y", self._y_coords), ("z", self._z_coords)):
            if len(c) < 2:
                raise ValueError(f"{name}_coords must have at least 2 points")
            if not np.all(np.diff(c) > 0):
                raise ValueError(f"{name}_coords must be monotonically increasing")
        self._dx = self._compute_spacing(self._x_coords)
        self._dy = self._compute_spacing(self._y_coords)
        self._dz = self._compute_spacing(self._z_coords)
        self._shape = (len(self._x_coords), len(self._y_coords), len(self._z_coords))

    @staticmethod
    def _compute_spacing(coords):
        """core/grid.py:217-235."""
        n = len(coords)
        spacing = np.zeros(n, dtype=np.float64)
        for i in range(1, n - 1):
            spacing[i] = (coords[i + 1] - coords[i - 1]) / 2
        spacing[0] = coords[1] - coords[0]
        spacing[-1] = coords[-1] - coords[-2]
        return spacing

    shape = property(lambda s: s._shape)
    dx = property(lambda s: s._dx)
    dy = property(lambda s: s._dy)
    dz = property(lambda s: s._dz)
    x_coords = property(lambda s: s._x_coords)
    y_coords = property(lambda s: s._y_coords)
    z_coords = property(lambda s: s._z_coords)

    @property
    def min_spacing(self) -> float:
        return float(min(np.min(self._dx), np.min(self._dy), np.min(self._dz)))

    @property
    def max_spacing(self) -> float:
        return float(max(np.max(self._dx), np.max(self._dy), np.max(self._dz)))

    @property
    def is_uniform(self) -> bool:
        return False

    @property
    def num_cells(self) -> int:
        return int(np.prod(self._shape))

    @property
    def stretch_ratio(self):
        return (float(np.max(self._dx) / np.min(self._dx)),
                float(np.max(self._dy) / np.min(self._dy)),
                float(np.max(self._dz) / np.min(self._dz)))

    def physical_extent(self):
        return (
            float(self._x_coords[-1] - self._x_coords[0] + self._dx[-1] / 2 + self._dx[0] / 2),
            float(self._y_coords[-1] - self._y_coords[0] + self._dy[-1] / 2 + self._dy[0] / 2),
            float(self._z_coords[-1] - self._z_coords[0] + self._dz[-1] / 2 + self._dz[0] / 2),
        )

    @classmethod
    def from_stretch(cls, shape, base_resolution: float, stretch_x: float = 1.0,
                     stretch_y: float = 1.0, stretch_z: float = 1.0, center_fine: bool = True):
        """Geometric growth per axis from the centre or from 0 (core/grid.py:325-407)."""
        nx, ny, nz = shape
        return cls(x_coords=cls._generate_stretched_coords(nx, base_resolution, stretch_x,
                                                           center_fine),
                   y_coords=cls._generate_stretched_coords(ny, base_resolution, stretch_y,
                                                           center_fine),
                   z_coords=cls._generate_stretched_coords(nz, base_resolution, stretch_z,
                                                           center_fine))

    @staticmethod
    def _generate_stretched_coords(n, base_dx, stretch, center_fine):
        if stretch == 1.0:
            return np.arange(n, dtype=np.float64) * base_dx + base_dx / 2
        if center_fine:
            n_half = n // 2
            sizes = base_dx * (stretch ** np.arange(n_half, dtype=np.float64))
            positions = np.cumsum(sizes) - sizes[0] / 2
            if n % 2 == 0:
                left = -positions[::-1] - sizes[::-1] / 2
                right = positions + sizes / 2
                coords = np.concatenate([left, right])
            else:
                left = -positions[::-1] - sizes[::-1] / 2
                center = np.array([0.0])
                right = positions[1:] + sizes[1:] / 2 if n_half > 0 else np.array([])
                coords = np.concatenate([left, center, right])
            coords = coords - coords[0] + base_dx / 2
        else:
            sizes = base_dx * (stretch ** np.arange(n, dtype=np.float64))
            coords = np.cumsum(sizes) - sizes / 2
        return coords

    @classmethod
    def from_regions(cls, x_regions, y_regions=None, z_regions=None):
        """Piecewise-constant resolution (core/grid.py:409-491)."""
        if y_regions is None:
            y_regions = x_regions
        if z_regions is None:
            z_regions = x_regions
        return cls(x_coords=cls._generate_region_coords(x_regions),
                   y_coords=cls._generate_region_coords(y_regions),
                   z_coords=cls._generate_region_coords(z_regions))

    @staticmethod
    def _generate_region_coords(regions):
        if not regions:
            raise ValueError("At least one region must be specified")
        coords_list: list = []
        for i, (start, end, resolution) in enumerate(regions):
            if end <= start:
                raise ValueError(f"Region {i}: end ({end}) must be > start ({start})")
            if resolution <= 0:
                raise ValueError(f"Region {i}: resolution must be positive")
            if i > 0:
                prev_end = regions[i - 1][1]
                if abs(start - prev_end) > 1e-10:
                    raise ValueError(f"Regions must be contiguous: region {i-1} ends at "
                                     f"{prev_end}, region {i} starts at {start}")
            n_cells = max(1, int(round((end - start) / resolution)))
            actual_resolution = (end - start) / n_cells
            region_coords = start + (np.arange(n_cells) + 0.5) * actual_resolution
            if coords_list and len(region_coords) > 0:
                if abs(region_coords[0] - coords_list[-1]) < actual_resolution / 2:
                    region_coords = region_coords[1:]
            coords_list.extend(region_coords.tolist())
        return np.array(coords_list, dtype=np.float64)

    def get_spacing_arrays_for_stencil(self) -> dict:
        """float32 inverse spacings: faces (centre distances, n-1) for the
        velocity update, cells (n) for the divergence (core/grid.py:493-532)."""
        return {
            "inv_dx_face": (1.0 / np.diff(self._x_coords)).astype(np.float32),
            "inv_dx_cell": (1.0 / self._dx).astype(np.float32),
            "inv_dy_face": (1.0 / np.diff(self._y_coords)).astype(np.float32),
            "inv_dy_cell": (1.0 / self._dy).astype(np.float32),
            "inv_dz_face": (1.0 / np.diff(self._z_coords)).astype(np.float32),
            "inv_dz_cell": (1.0 / self._dz).astype(np.float32),
        }
