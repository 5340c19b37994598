"""Membrane sources: a waveform injected over a disc or rectangle of one grid
plane, weighted by a clamped-membrane mode shape (core/solver.py:210-755 of
rjwalters/strata-fdtd).

The weights are computed on the host with the reference's NumPy / SciPy
expressions (Bessel J_m modes for a disc, sin x sin for a rectangle,
normalised to a maximum of 1); the GPU adds value x weight to the pressure
(or to the normal velocity) of the masked air cells after each step, in
FP64 with one rounding, as NumPy's ``p[mask] += value * weights[mask]``
does (core/solver.py:2389-2412).
"""
from __future__ import annotations

import warnings
from dataclasses import dataclass, field
from typing import Literal

import numpy as np
from scipy.special import j0, jn_zeros, jv


@dataclass
class MembraneSource:
    """Spatially distributed source on the grid plane nearest ``center``
    (metres) perpendicular to ``normal_axis``; ``waveform`` is any object
    with ``.waveform(t, dt)``; ``injection_type`` 'pressure' or 'velocity'."""

    center: tuple[float, float, float]
    normal_axis: Literal["x", "y", "z"]
    waveform: object
    mode: tuple[int, int] = (0, 1)
    injection_type: Literal["pressure", "velocity"] = "pressure"
    source_type: Literal["membrane"] = field(default="membrane", init=False)
    _cached_weights: np.ndarray | None = field(default=None, repr=False, init=False)
    _cached_mask: np.ndarray | None = field(default=None, repr=False, init=False)

    def mode_shape(self, r, theta):
        raise NotImplementedError("Subclasses must implement mode_shape()")

    def get_injection_mask(self, grid):
        raise NotImplementedError("Subclasses must implement get_injection_mask()")

    def get_injection_weights(self, grid):
        raise NotImplementedError("Subclasses must implement get_injection_weights()")

    def _plane_index(self, grid) -> int:
        c = {"x": (grid.x_coords, self.center[0]), "y": (grid.y_coords, self.center[1]),
             "z": (grid.z_coords, self.center[2])}[self.normal_axis]
        return int(np.argmin(np.abs(c[0] - c[1])))

    def _in_plane_offsets(self, grid):
        """Offsets (a, b) from the centre along the two in-plane axes, as 3-D
        meshgrid arrays, and the plane index (core/solver.py:290-336)."""
        x, y, z = np.meshgrid(grid.x_coords, grid.y_coords, grid.z_coords, indexing="ij")
        cx, cy, cz = self.center
        if self.normal_axis == "z":
            return x - cx, y - cy, self._plane_index(grid)
        if self.normal_axis == "y":
            return x - cx, z - cz, self._plane_index(grid)
        return y - cy, z - cz, self._plane_index(grid)

    def _plane_mask(self, grid, inside) -> np.ndarray:
        mask = np.zeros(grid.shape, dtype=bool)
        k = self._plane_index(grid)
        if self.normal_axis == "z":
            mask[:, :, k] = inside[:, :, k]
        elif self.normal_axis == "y":
            mask[:, k, :] = inside[:, k, :]
        else:
            mask[k, :, :] = inside[k, :, :]
        return mask

    def _check_grid_alignment(self, grid) -> None:
        """Warn when the centre lies more than half a cell off the plane
        (core/solver.py:338-369)."""
        ax = "xyz".index(self.normal_axis)
        coords = (grid.x_coords, grid.y_coords, grid.z_coords)[ax]
        spacing_arr = (grid.dx, grid.dy, grid.dz)[ax]
        k = self._plane_index(grid)
        offset = abs(coords[k] - self.center[ax])
        spacing = spacing_arr[k] if hasattr(spacing_arr, "__getitem__") else grid.min_spacing
        if offset > 0.5 * spacing:
            warnings.warn(f"MembraneSource center {self.center} is {offset:.4f}m "
                          f"({offset/spacing:.1f} cells) off-grid in {self.normal_axis}-direction. "
                          "Source will be placed at nearest grid plane.", stacklevel=3)


@dataclass(kw_only=True)
class CircularMembraneSource(MembraneSource):
    """Disc of ``radius`` clamped at its edge: |J_m(alpha_mn r/a) cos(m theta)|
    normalised to 1, alpha_mn the n-th zero of J_m (core/solver.py:372-503)."""

    radius: float
    _alpha: float = field(default=0.0, repr=False, init=False)

    _ZEROS = {(0, 1): 2.4048255576957727, (0, 2): 5.5200781102863115,
              (1, 1): 3.8317059702075125, (1, 2): 7.0155866698156190,
              (2, 1): 5.1356223018406826, (2, 2): 8.4172441403998649}

    def __post_init__(self) -> None:
        m, n = self.mode
        if m < 0:
            raise ValueError(f"Azimuthal mode m must be non-negative, got {m}")
        if n < 1:
            raise ValueError(f"Radial mode n must be positive, got {n}")
        self._alpha = self._ZEROS.get((m, n)) or jn_zeros(m, n)[-1]

    def _polar(self, grid):
        a, b, k = self._in_plane_offsets(grid)
        return np.sqrt(a**2 + b**2), np.arctan2(b, a), k

    def mode_shape(self, r, theta):
        m, _ = self.mode
        rho = r / self.radius
        if m == 0:
            shape = j0(self._alpha * rho)
        else:
            shape = jv(m, self._alpha * rho) * np.cos(m * theta)
        shape = np.where(rho <= 1.0, shape, 0.0)
        shape = np.abs(shape)
        max_val = np.max(shape)
        return shape / max_val if max_val > 1e-10 else np.zeros_like(shape)

    def get_injection_mask(self, grid):
        r, _, _ = self._polar(grid)
        return self._plane_mask(grid, r <= self.radius)

    def get_injection_weights(self, grid):
        self._check_grid_alignment(grid)
        r, theta, _ = self._polar(grid)
        weights = np.zeros(grid.shape, dtype=np.float64)
        mask = self.get_injection_mask(grid)
        weights[mask] = self.mode_shape(r[mask], theta[mask])
        return weights


@dataclass(kw_only=True)
class RectangularMembraneSource(MembraneSource):
    """Rectangle ``size`` = (width, height) in the membrane plane, clamped at
    its edges: |sin(m pi (u/Lx + 1/2)) sin(n pi (v/Ly + 1/2))| normalised to 1
    (core/solver.py:505-755)."""

    size: tuple[float, float]
    mode: tuple[int, int] = (1, 1)

    def __post_init__(self) -> None:
        m, n = self.mode
        if m < 1:
            raise ValueError(f"Mode index m must be >= 1, got {m}")
        if n < 1:
            raise ValueError(f"Mode index n must be >= 1, got {n}")

    def mode_shape(self, u, v):
        m, n = self.mode
        Lx, Ly = self.size
        shape = np.sin(m * np.pi * (u / Lx + 0.5)) * np.sin(n * np.pi * (v / Ly + 0.5))
        inside = (np.abs(u) <= Lx / 2) & (np.abs(v) <= Ly / 2)
        shape = np.abs(np.where(inside, shape, 0.0))
        max_val = np.max(shape)
        return shape / max_val if max_val > 1e-10 else np.zeros_like(shape)

    def get_injection_mask(self, grid):
        u, v, _ = self._in_plane_offsets(grid)
        Lx, Ly = self.size
        return self._plane_mask(grid, (np.abs(u) <= Lx / 2) & (np.abs(v) <= Ly / 2))

    def get_injection_weights(self, grid):
        self._check_grid_alignment(grid)
        u, v, _ = self._in_plane_offsets(grid)
        weights = np.zeros(grid.shape, dtype=np.float64)
        mask = self.get_injection_mask(grid)
        weights[mask] = self.mode_shape(u[mask], v[mask])
        return weights
