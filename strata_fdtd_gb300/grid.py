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


def _axis_coords(values, axis: str) -> np.ndarray:
    """One axis's cell centres as a flat float64 array: two or more of them,
    strictly increasing."""
    c = np.asarray(values, dtype=np.float64).ravel()
    if c.size < 2:
        raise ValueError(f"{axis}_coords: a nonuniform axis needs at least 2 cell centres")
    if np.any(c[1:] <= c[:-1]):
        raise ValueError(f"{axis}_coords: cell centres must be monotonically increasing "
                         "(strictly)")
    return c


def _cell_widths(c: np.ndarray) -> np.ndarray:
    """Width of each cell: half the distance between its neighbours' centres
    inside, the distance to the one neighbour at either end."""
    w = np.empty_like(c)
    w[1:-1] = (c[2:] - c[:-2]) / 2
    w[0], w[-1] = c[1] - c[0], c[-1] - c[-2]
    return w


def _geometric_centres(n: int, h0: float, ratio: float, from_centre: bool) -> np.ndarray:
    """Centres of n cells whose widths grow by ``ratio`` per cell: outward
    from the middle (mirrored halves, an extra centre cell for odd n) or
    from the low end; h0 is the smallest width and the first centre sits at
    h0 / 2.  A ratio of 1 gives the uniform centres."""
    if ratio == 1.0:
        return np.arange(n, dtype=np.float64) * h0 + h0 / 2
    if not from_centre:
        widths = h0 * ratio ** np.arange(n, dtype=np.float64)
        return np.cumsum(widths) - widths / 2
    widths = h0 * ratio ** np.arange(n // 2, dtype=np.float64)
    outer = (np.cumsum(widths) - widths[0] / 2) + widths / 2  # one half, mirrored below
    mirrored = -outer[::-1]
    c = (np.concatenate([mirrored, outer]) if n % 2 == 0
         else np.concatenate([mirrored, [0.0], outer[1:]]))
    return (c - c[0]) + h0 / 2


def _piecewise_centres(regions) -> np.ndarray:
    """Centres of consecutive (start, end, resolution) regions: each region
    holds round(length / resolution) (at least one) equal cells; a region's
    first centre is dropped when it lies within half a cell of the previous
    region's last one."""
    regions = list(regions or [])
    if not regions:
        raise ValueError("from_regions: give at least one (start, end, resolution) region")
    for n, (lo, hi, res) in enumerate(regions):
        if not hi > lo:
            raise ValueError(f"from_regions: region {n} has end {hi} not above start {lo}")
        if not res > 0:
            raise ValueError(f"from_regions: region {n}: resolution must be positive, got {res}")
        if n and abs(lo - regions[n - 1][1]) > 1e-10:
            raise ValueError(f"from_regions: regions must be contiguous; region {n} starts "
                             f"at {lo}, region {n - 1} ends at {regions[n - 1][1]}")
    out: list = []
    for lo, hi, res in regions:
        cells = max(1, int(round((hi - lo) / res)))
        h = (hi - lo) / cells
        centres = lo + (np.arange(cells) + 0.5) * h
        if out and abs(centres[0] - out[-1]) < h / 2:
            centres = centres[1:]
        out.extend(centres.tolist())
    return np.array(out, dtype=np.float64)


class NonuniformGrid:
    """A grid with its own cell centres per axis (core/grid.py:148-532 of
    rjwalters/strata-fdtd): cell widths from the centres (``_cell_widths``),
    face spacings as the centre distances, geometric and piecewise
    generators, and the float32 inverse spacings the kernels take.  Every
    value is the reference's FP64 number, which the nonuniform parity cases
    rely on."""

    def __init__(self, x_coords, y_coords, z_coords):
        self._c = tuple(_axis_coords(v, a) for v, a in zip((x_coords, y_coords, z_coords), "xyz"))
        self._w = tuple(_cell_widths(c) for c in self._c)

    shape = property(lambda s: tuple(c.size for c in s._c))
    x_coords = property(lambda s: s._c[0])
    y_coords = property(lambda s: s._c[1])
    z_coords = property(lambda s: s._c[2])
    dx = property(lambda s: s._w[0])
    dy = property(lambda s: s._w[1])
    dz = property(lambda s: s._w[2])

    @property
    def min_spacing(self) -> float:
        return float(min(w.min() for w in self._w))

    @property
    def max_spacing(self) -> float:
        return float(max(w.max() for w in self._w))

    @property
    def is_uniform(self) -> bool:
        return False

    @property
    def num_cells(self) -> int:
        return int(np.prod(self.shape))

    @property
    def stretch_ratio(self):
        return tuple(float(w.max() / w.min()) for w in self._w)

    def physical_extent(self):
        """Span of each axis from the low face of its first cell to the high
        face of its last."""
        return tuple(float(c[-1] - c[0] + w[-1] / 2 + w[0] / 2) for c, w in zip(self._c, self._w))

    @classmethod
    def from_stretch(cls, shape, base_resolution: float, stretch_x: float = 1.0,
                     stretch_y: float = 1.0, stretch_z: float = 1.0, center_fine: bool = True):
        """Widths growing geometrically per axis, finest at the centre or at
        the low end (core/grid.py:325-407)."""
        ratios = (stretch_x, stretch_y, stretch_z)
        return cls(*(_geometric_centres(int(n), base_resolution, r, center_fine)
                     for n, r in zip(shape, ratios)))

    @classmethod
    def from_regions(cls, x_regions, y_regions=None, z_regions=None):
        """Piecewise-constant resolution per axis; y and z default to the x
        regions (core/grid.py:409-491)."""
        return cls(*(_piecewise_centres(r if r is not None else x_regions)
                     for r in (x_regions, y_regions, z_regions)))

    def get_spacing_arrays_for_stencil(self) -> dict:
        """float32 inverse spacings: faces (centre distances, n-1) for the
        velocity update, cells (n) for the divergence (core/grid.py:493-532)."""
        out = {}
        for a, c, w in zip("xyz", self._c, self._w):
            out[f"inv_d{a}_face"] = (1.0 / np.diff(c)).astype(np.float32)
            out[f"inv_d{a}_cell"] = (1.0 / w).astype(np.float32)
        return out
