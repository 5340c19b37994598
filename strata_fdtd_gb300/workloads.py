"""The benchmark workloads, built through the public API.

quick_start_100   100^3, 1 mm, air (c 343, rho 1.204), courant 0.5, PML 10,
                  1 kHz pulse at (50,50,50), probe at (75,50,50), 1000 steps --
                  the reference's README quick start with its real API.
enclosure_400     400^3, 1 mm, PML 16, rigid walls voxelised from a
                  200 x 120 x 300 mm box enclosure with 12 mm walls and a
                  radius-25 mm, 80 mm port through the z-min wall, centred at
                  (0.2, 0.2, 0.2) m; 2 kHz pulse at the cavity centre; 8
                  probes at seeded random air cells outside the walls and the
                  PML; 4000 steps.
"""
from __future__ import annotations

import numpy as np

from .boundaries import PML
from .grid import UniformGrid
from .sdf import Box, Cylinder, Difference
from .solver import FDTDSolver, GaussianPulse

C_AIR, RHO_AIR = 343.0, 1.204


def enclosure_solid():
    centre = (0.2, 0.2, 0.2)
    outer = Box(center=centre, size=(0.2, 0.12, 0.3))
    inner = Box(center=centre, size=(0.176, 0.096, 0.276))
    z0 = 0.2 - 0.15
    port = Cylinder(p1=(0.2, 0.2, z0), p2=(0.2, 0.2, z0 + 0.08), radius=0.025)
    return Difference(outer, inner, port)


def enclosure_probes(geometry, pml_depth=16, n=8, seed=0):
    """Seeded air cells outside the enclosure's bounding cells and the PML
    (cell indices for the 0.4 m cube at any resolution)."""
    rng = np.random.default_rng(seed)
    size = geometry.shape[0]
    res = 0.4 / size
    lo_box = np.floor(np.array([0.1, 0.14, 0.05]) / res).astype(int) - 1
    hi_box = np.ceil(np.array([0.3, 0.26, 0.35]) / res).astype(int) + 1
    out = []
    while len(out) < n:
        c = rng.integers(pml_depth, size - pml_depth, size=3)
        if (np.all(c >= lo_box) and np.all(c < hi_box)) or not geometry[tuple(c)]:
            continue
        out.append(tuple(int(v) for v in c))
    return out


def enclosure(n=400, amplitude=1.0, **kw) -> FDTDSolver:
    """The enclosure workload on an n^3 grid over the same 0.4 m cube
    (n = 400: 1 mm cells, PML 16; smaller n for profiling runs)."""
    res = 1e-3 if n == 400 else 0.4 / n
    pml = 16 if n == 400 else max(4, round(16 * n / 400))
    s = FDTDSolver(grid=UniformGrid((n, n, n), res), c=C_AIR, rho=RHO_AIR, courant=0.5,
                   backend="native", **kw)
    s.add_boundary(PML(depth=pml))
    s.set_geometry_sdf(enclosure_solid())
    s.add_source(GaussianPulse(position=(n // 2, n // 2, n // 2), frequency=2000.0,
                               amplitude=amplitude))
    for q, pos in enumerate(enclosure_probes(s.geometry, pml_depth=pml)):
        s.add_probe(f"probe{q}", pos)
    return s


def enclosure_400(amplitude=1.0, **kw) -> FDTDSolver:
    return enclosure(400, amplitude, **kw)


def quick_start_100(**kw) -> FDTDSolver:
    s = FDTDSolver(grid=UniformGrid((100, 100, 100), 1e-3), c=C_AIR, rho=RHO_AIR, courant=0.5,
                   backend="native", **kw)
    s.add_boundary(PML(depth=10))
    s.add_source(GaussianPulse(position=(50, 50, 50), frequency=1000.0, amplitude=1.0))
    s.add_probe("output", (75, 50, 50))
    return s
