"""Helmholtz resonators as SDF trees (geometry/resonator.py:59-468 of
rjwalters/strata-fdtd).  Construction mirrors the reference's NumPy
arithmetic so the cavity and neck constants are bit-identical; evaluation is
the GPU voxeliser's."""
from __future__ import annotations

import numpy as np

from .sdf import Box, Cylinder, SDFPrimitive, Sphere, Union

SPEED_OF_SOUND = 343.0


class HelmholtzResonator(SDFPrimitive):
    """Cavity (box / sphere / cylinder) plus a cylindrical neck."""

    def __init__(self, position, cavity_shape="box", cavity_size=(0.03, 0.03, 0.03),
                 neck_length=0.01, neck_radius=0.005, neck_direction=(0.0, 0.0, 1.0),
                 opening_type="unflanged"):
        self.position = np.asarray(position, dtype=np.float64)
        nd = np.asarray(neck_direction, dtype=np.float64)
        norm = np.linalg.norm(nd)
        if norm < 1e-10:
            raise ValueError("neck_direction cannot be zero vector")
        self.neck_direction = nd / norm
        if neck_length <= 0:
            raise ValueError(f"neck_length must be positive, got {neck_length}")
        if neck_radius <= 0:
            raise ValueError(f"neck_radius must be positive, got {neck_radius}")
        self.cavity_shape = cavity_shape
        self.cavity_size = cavity_size
        self.neck_length = neck_length
        self.neck_radius = neck_radius
        self.opening_type = opening_type
        self._build_geometry()

    def _build_geometry(self):
        """resonator.py:142-185."""
        def sizes(n, names):
            got = tuple(self.cavity_size)
            if len(got) != n:
                raise ValueError(f"a {self.cavity_shape} cavity requires {n} size "
                                 f"parameter{'s' if n > 1 else ''} ({names}), got {len(got)}")
            if any(v <= 0 for v in got):
                raise ValueError(f"cavity sizes must be positive, got {got}")
            return got

        if self.cavity_shape == "box":
            self._cavity = Box(center=tuple(self.position), size=sizes(3, "x, y, z"))
        elif self.cavity_shape == "sphere":
            self._cavity = Sphere(center=tuple(self.position), radius=sizes(1, "radius")[0])
        elif self.cavity_shape == "cylinder":
            r, length = sizes(2, "radius, length")
            axis = self.neck_direction * length
            self._cavity = Cylinder(p1=tuple(self.position - axis / 2),
                                    p2=tuple(self.position + axis / 2), radius=r)
        else:
            raise ValueError(f"Unknown cavity_shape: {self.cavity_shape}")
        start = self._cavity_surface_point()
        end = start + self.neck_direction * self.neck_length
        self._neck = Cylinder(p1=tuple(start), p2=tuple(end), radius=self.neck_radius)
        self._combined = Union(self._cavity, self._neck)

    def _cavity_surface_point(self):
        """resonator.py:187-207."""
        if self.cavity_shape == "box":
            half = np.array(self.cavity_size, dtype=np.float64) / 2
            t = np.min(half / (np.abs(self.neck_direction) + 1e-10))
            return self.position + self.neck_direction * t
        if self.cavity_shape == "sphere":
            return self.position + self.neck_direction * self.cavity_size[0]
        return self.position + self.neck_direction * (self.cavity_size[1] / 2)

    def _emit(self, prog):
        self._combined._emit(prog)

    @property
    def bounding_box(self):
        return self._combined.bounding_box

    @property
    def cavity_volume(self) -> float:
        if self.cavity_shape == "box":
            return float(np.prod(self.cavity_size))
        if self.cavity_shape == "sphere":
            return (4 / 3) * np.pi * self.cavity_size[0] ** 3
        r, length = self.cavity_size
        return np.pi * r**2 * length

    @property
    def neck_area(self) -> float:
        return np.pi * self.neck_radius**2

    @property
    def effective_neck_length(self) -> float:
        k = 0.85 if self.opening_type == "flanged" else 0.6
        return self.neck_length + 2 * k * self.neck_radius

    @property
    def resonant_frequency(self) -> float:
        S, V, L = self.neck_area, self.cavity_volume, self.effective_neck_length
        return float((SPEED_OF_SOUND / (2 * np.pi)) * np.sqrt(S / (V * L)))

    @property
    def quality_factor(self) -> float:
        """The reference's placeholder Q estimate: a constant 10
        (resonator.py:281-297; a real Q needs the neck's viscothermal
        losses)."""
        return 10.0


def helmholtz_array(region, frequency_range, n_resonators, spacing="log", cavity_shape="box",
                    neck_length=0.01, neck_radius=0.003):
    """Detuned resonators laid out on a grid inside ``region``'s bounding box
    (resonator.py:300-468)."""
    f_min, f_max = frequency_range
    if f_min <= 0 or f_max < f_min:
        raise ValueError(f"Invalid frequency range: ({f_min}, {f_max})")
    if n_resonators < 1:
        raise ValueError(f"n_resonators must be >= 1, got {n_resonators}")
    if spacing == "log":
        freqs = np.geomspace(f_min, f_max, n_resonators)
    elif spacing == "linear":
        freqs = np.linspace(f_min, f_max, n_resonators)
    else:
        raise ValueError(f"spacing must be 'log' or 'linear', got {spacing}")
    bb_min, bb_max = region.bounding_box
    size = bb_max - bb_min
    out = []
    n = int(np.ceil(np.cbrt(n_resonators)))
    for i, f in enumerate(freqs):
        S = np.pi * neck_radius**2
        L_eff = neck_length + 1.2 * neck_radius
        V = S / (L_eff * (2 * np.pi * f / SPEED_OF_SOUND) ** 2)
        if cavity_shape == "box":
            side = np.cbrt(V)
            cav = (side, side, side)
        elif cavity_shape == "sphere":
            cav = (np.cbrt(3 * V / (4 * np.pi)),)
        else:
            r = np.cbrt(V / (2 * np.pi))
            cav = (r, 2 * r)
        ix, iy, iz = i % n, (i // n) % n, i // (n * n)
        eff = size * (1 - 2 * 0.05)
        pos = bb_min + size * 0.05 + (eff / n) * np.array([ix + 0.5, iy + 0.5, iz + 0.5])
        out.append(HelmholtzResonator(position=pos, cavity_shape=cavity_shape, cavity_size=cav,
                                      neck_length=neck_length, neck_radius=neck_radius,
                                      neck_direction=(0, 0, 1)))
    return out
