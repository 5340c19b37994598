"""Curved paths for swept geometry (geometry/paths.py of rjwalters/strata-fdtd).

Sampled on the host with the reference's NumPy calls, so the vertices the GPU
voxeliser receives for ``SpiralHorn`` and ``HelicalTube`` are the reference's
vertices; ``distance_to_polyline`` is the host restatement of the distance
those shapes take on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SpiralPath:
    """Logarithmic (r = r0 exp(k theta)) or Archimedean (r = r0 + k theta)
    spiral in the xy plane from ``inner_radius`` to ``outer_radius`` over
    ``turns`` turns about ``center`` (paths.py:30-134)."""

    center: object
    inner_radius: float
    outer_radius: float
    turns: float
    spiral_type: str = "logarithmic"

    def __post_init__(self) -> None:
        self.center = np.asarray(self.center, dtype=np.float64)
        if self.center.shape != (2,):
            raise ValueError(f"center must be 2D point, got shape {self.center.shape}")
        if self.inner_radius <= 0:
            raise ValueError(f"inner_radius must be positive, got {self.inner_radius}")
        if self.outer_radius <= self.inner_radius:
            raise ValueError(f"outer_radius ({self.outer_radius}) must be > inner_radius "
                             f"({self.inner_radius})")
        if self.turns <= 0:
            raise ValueError(f"turns must be positive, got {self.turns}")
        if self.spiral_type not in ("logarithmic", "archimedean"):
            raise ValueError("spiral_type must be 'logarithmic' or 'archimedean', "
                             f"got '{self.spiral_type}'")

    def sample_points(self, n_points: int = 100) -> np.ndarray:
        """(n, 2) points at angles evenly spaced from 0 to 2 pi turns."""
        if n_points < 2:
            raise ValueError(f"n_points must be >= 2, got {n_points}")
        sweep = 2 * np.pi * self.turns
        theta = np.linspace(0, sweep, n_points)
        if self.spiral_type == "logarithmic":
            k = np.log(self.outer_radius / self.inner_radius) / sweep
            r = self.inner_radius * np.exp(k * theta)
        else:
            k = (self.outer_radius - self.inner_radius) / sweep
            r = self.inner_radius + k * theta
        return np.stack([self.center[0] + r * np.cos(theta),
                         self.center[1] + r * np.sin(theta)], axis=1)

    @property
    def total_length(self) -> float:
        """Arc length of a 1000-point sampling."""
        pts = self.sample_points(1000)
        return float(np.sum(np.linalg.norm(np.diff(pts, axis=0), axis=1)))


@dataclass
class HelixPath:
    """Helix about the z axis through ``center`` (its bottom), of ``radius``,
    rising ``pitch`` per turn over ``turns`` turns (paths.py:137-223)."""

    center: object
    radius: float
    pitch: float
    turns: float

    def __post_init__(self) -> None:
        self.center = np.asarray(self.center, dtype=np.float64)
        if self.center.shape != (3,):
            raise ValueError(f"center must be 3D point, got shape {self.center.shape}")
        for name in ("radius", "pitch", "turns"):
            if getattr(self, name) <= 0:
                raise ValueError(f"{name} must be positive, got {getattr(self, name)}")

    def sample_points(self, n_points: int = 100) -> np.ndarray:
        """(n, 3) points at angles evenly spaced from 0 to 2 pi turns."""
        if n_points < 2:
            raise ValueError(f"n_points must be >= 2, got {n_points}")
        theta = np.linspace(0, 2 * np.pi * self.turns, n_points)
        return np.stack([self.center[0] + self.radius * np.cos(theta),
                         self.center[1] + self.radius * np.sin(theta),
                         self.center[2] + (theta / (2 * np.pi)) * self.pitch], axis=1)

    @property
    def total_length(self) -> float:
        return float(self.turns * np.sqrt((2 * np.pi * self.radius) ** 2 + self.pitch ** 2))

    @property
    def total_height(self) -> float:
        return float(self.turns * self.pitch)


def distance_to_polyline(points, polyline) -> np.ndarray:
    """Distance from each of (N, d) points to the polyline of (M, d) vertices:
    the minimum over its segments of the distance to the closest point on
    the segment (a segment shorter than 1e-7 counts as its first vertex)."""
    points = np.asarray(points, dtype=np.float64)
    polyline = np.asarray(polyline, dtype=np.float64)
    if points.shape[1] != polyline.shape[1]:
        raise ValueError(f"Dimension mismatch: points are {points.shape[1]}D, "
                         f"polyline is {polyline.shape[1]}D")
    if polyline.shape[0] < 2:
        raise ValueError(f"Polyline must have >= 2 vertices, got {polyline.shape[0]}")
    best = np.full(points.shape[0], np.inf)
    for a, b in zip(polyline[:-1], polyline[1:]):
        seg = b - a
        ll = np.dot(seg, seg)
        if ll < 1e-14:
            d = np.linalg.norm(points - a, axis=1)
        else:
            t = np.clip(np.dot(points - a, seg) / ll, 0, 1)
            d = np.linalg.norm(points - (a + t[:, None] * seg), axis=1)
        best = np.minimum(best, d)
    return best


def distance_to_helix(points, center, radius: float, pitch: float, turns: float) -> np.ndarray:
    """Distance from (N, 3) points to the helix of ``HelixPath``, taken as
    the polyline through max(100, int(50 turns)) of its samples
    (geometry/paths.py:296-344)."""
    points = np.asarray(points, dtype=np.float64)
    center = np.asarray(center, dtype=np.float64)
    if points.ndim != 2 or points.shape[1] != 3:
        raise ValueError(f"points must be Nx3 array, got shape {points.shape}")
    if center.shape != (3,):
        raise ValueError(f"center must be 3D point, got shape {center.shape}")
    helix = HelixPath(center=center, radius=radius, pitch=pitch, turns=turns)
    return distance_to_polyline(points, helix.sample_points(max(100, int(50 * turns))))
