"""Material regions assigned from SDF geometry (geometry/material_assignment.py
of rjwalters/strata-fdtd), voxelised on the GPU.

``MaterializedGeometry`` keeps the reference's interface: an SDF whose
inside is air, a default material (id 0), and regions added in order with
``set_material`` (ids 1, 2, ... in assignment order, later regions
overriding earlier ones, only inside air).  ``voxelize_with_materials``
runs the geometry program and every region program per cell in one kernel
(``sf_voxelize_materials``, FP64, the reference's SDF arithmetic), so the
mask and the material ids are the reference's NumPy result bit for bit and
neither an intermediate mask per region nor a host pass is needed.
``FDTDSolver.set_geometry`` accepts it (core/solver.py:1715-1760).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native
from .sdf import Box, SDFPrimitive


class MaterializedGeometry:
    """An SDF geometry (inside = air) with ordered material regions.

    geometry          SDF primitive whose inside is the air / material volume
    default_material  material of cells no region claims (id 0); AIR_20C
                      when omitted
    """

    def __init__(self, geometry: SDFPrimitive, default_material=None):
        if default_material is None:
            from .materials import AIR_20C

            default_material = AIR_20C
        self.geometry = geometry
        self.default_material = default_material
        self._material_regions: list = []  # (region SDF, material, id)
        self._material_id_counter = 1      # 0 is the default material

    def set_material(self, region: SDFPrimitive, material) -> int:
        """Assign ``material`` to the air cells inside ``region``; returns its
        id (1-255).  Later assignments win where regions overlap."""
        if self._material_id_counter > 255:
            raise ValueError("Maximum of 255 material regions exceeded")
        mid = self._material_id_counter
        self._material_id_counter += 1
        self._material_regions.append((region, material, mid))
        return mid

    def _programs(self):
        nodes, off, ids = [], [0], []
        for prog_owner in [self.geometry] + [r for r, _, _ in self._material_regions]:
            prog: list = []
            prog_owner._emit(prog)
            nodes.extend(prog)
            off.append(len(nodes))
        ids = [mid for _, _, mid in self._material_regions]
        return ((_native.SfSdfNode * len(nodes))(*nodes), (ctypes.c_int32 * len(off))(*off),
                (ctypes.c_uint8 * max(1, len(ids)))(*ids), len(ids))

    def voxelize_with_materials_device(self, grid, stream=None):
        """(geometry, material_ids) as torch.uint8 CUDA tensors of grid.shape
        (geometry 1 = air)."""
        import torch

        nx, ny, nz = grid.shape
        geom = torch.empty((nx, ny, nz), dtype=torch.uint8, device="cuda")
        mat = torch.empty((nx, ny, nz), dtype=torch.uint8, device="cuda")
        nodes, off, ids, n = self._programs()
        st = (stream or torch.cuda.current_stream()).cuda_stream
        coords = None
        keep = None
        if not getattr(grid, "is_uniform", True):  # the nonuniform grid's own cell centres
            keep = [np.ascontiguousarray(c, dtype=np.float64)
                    for c in (grid.x_coords, grid.y_coords, grid.z_coords)]
            coords = (ctypes.c_void_p * 3)(*[c.ctypes.data for c in keep])
        res = float(grid.min_spacing) if coords is None else 0.0
        _native.check(_native.load().sf_voxelize_materials(
            ctypes.addressof(nodes), ctypes.addressof(off), n, ctypes.addressof(ids), nx, ny, nz,
            res, coords, geom.data_ptr(), mat.data_ptr(), st), "sf_voxelize_materials")
        del keep
        return geom, mat

    def voxelize_with_materials(self, grid):
        """(geometry_mask bool, material_ids uint8) NumPy arrays of grid.shape
        (material_assignment.py:133-171)."""
        geom, mat = self.voxelize_with_materials_device(grid)
        return geom.cpu().numpy().astype(bool), mat.cpu().numpy()

    def get_material_table(self) -> dict:
        table = {0: self.default_material}
        for _, material, mid in self._material_regions:
            table[mid] = material
        return table

    def material_count(self) -> int:
        return len(self._material_regions) + 1

    def __repr__(self) -> str:
        return (f"MaterializedGeometry(geometry={type(self.geometry).__name__}, "
                f"materials={self.material_count()})")


@dataclass
class MaterialVolume:
    """A box-shaped material region from (min_corner, max_corner) bounds or a
    centre and size (material_assignment.py:205-348)."""

    material: object
    bounds: tuple | None = None
    center: tuple | None = None
    size: tuple | None = None

    def __post_init__(self):
        if self.bounds is None:
            if self.center is None or self.size is None:
                raise ValueError("Must provide either bounds or (center, size)")
            c = np.array(self.center, dtype=np.float64)
            half = np.array(self.size, dtype=np.float64) / 2
            self.bounds = (c - half, c + half)
            return
        if not isinstance(self.bounds, tuple) or len(self.bounds) != 2:
            raise ValueError("bounds must be tuple of (min_corner, max_corner)")
        lo, hi = (np.asarray(b, dtype=np.float64) for b in self.bounds)
        if lo.shape != (3,) or hi.shape != (3,):
            raise ValueError("bounds corners must be 3-element arrays")
        if np.any(lo >= hi):
            raise ValueError("min_corner must be less than max_corner in all dimensions")
        self.bounds = (lo, hi)

    @property
    def region(self) -> Box:
        lo, hi = self.bounds
        return Box(min_corner=tuple(lo), max_corner=tuple(hi))

    @classmethod
    def from_center_size(cls, center, size, material) -> "MaterialVolume":
        return cls(material=material, center=center, size=size)

    @classmethod
    def from_corners(cls, min_corner, max_corner, material) -> "MaterialVolume":
        return cls(material=material, bounds=(np.asarray(min_corner, dtype=np.float64),
                                              np.asarray(max_corner, dtype=np.float64)))
