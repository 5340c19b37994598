"""Golden-vector cases, written once against the reference API.

Each case is plain data plus a builder that drives any module exposing the
reference's solver API (``FDTDSolver``, ``UniformGrid``, ``PML``,
``GaussianPulse``, the SDF classes and the material classes).  The same
builder runs the reference itself (``make_golden.py``, in a container where
the reference tree exists) and ``strata_fdtd_gb300`` (the GPU tests), so a
golden fixture and its replay cannot drift apart.

Reference API used (paths relative to src/strata_fdtd/ of
rjwalters/strata-fdtd): FDTDSolver.__init__ core/solver.py:1507-1518,
add_boundary :1983, set_geometry :1682, add_source :1782, add_probe :1843,
register_material :2836, set_material_box :2900, PML boundaries/_boundaries.py:125,
GaussianPulse core/solver.py:152, SDF geometry/sdf.py, HelmholtzResonator
geometry/resonator.py:59, Pole/SimpleMaterial materials/base.py:55,509.
"""
from __future__ import annotations

import json
import os

import numpy as np

AIR = dict(c=343.0, rho=1.204)


def _mask_blocks(shape, seed, n_boxes=2, n_spheres=1):
    """Seeded solid blocks and balls, True = air (the reference convention)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    g = np.ones(shape, dtype=bool)
    for _ in range(n_boxes):
        lo = [int(rng.integers(1, n - 4)) for n in shape]
        hi = [min(n, l + int(rng.integers(2, max(3, n // 3)))) for l, n in zip(lo, shape)]
        g[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = False
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for _ in range(n_spheres):
        c = [int(rng.integers(2, n - 2)) for n in shape]
        r = int(rng.integers(2, max(3, min(shape) // 4)))
        g[(ii - c[0]) ** 2 + (jj - c[1]) ** 2 + (kk - c[2]) ** 2 <= r * r] = False
    return g


def gain_07_03(theta):
    """Custom microphone pattern of the directional golden case."""
    return 0.7 + 0.3 * np.cos(theta)


# --------------------------------------------------------------------------
# Plain path: reference FDTDSolver(backend="native") step for step.
# source tuple: (kind, position, frequency, amplitude); a plane position is a
# dict {"axis": a, "index": n}.
PLAIN_CASES = {
    "c1_tiny": dict(
        shape=(32, 32, 32), res=1e-3, courant=0.5, pml=dict(depth=6),
        sources=[("point", (16, 16, 16), 20000.0, 1.0)],
        probes=[("out", (24, 16, 16)), ("src", (16, 16, 16))],
        steps=200, store_fields=True,
    ),
    "blocks_odd": dict(
        shape=(17, 23, 29), res=1e-3, courant=0.5, pml=dict(depth=3),
        geometry=dict(kind="blocks", seed=3),
        sources=[("point", (3, 4, 5), 30000.0, 2.0), ("point", (3, 4, 5), 15000.0, -0.5)],
        probes=[("a", (8, 11, 14)), ("b", (1, 20, 27)), ("c", (16, 22, 28))],
        steps=150, store_fields=True,
    ),
    "plane_x_pml_x": dict(
        shape=(24, 20, 16), res=1e-3, courant=0.5, pml=dict(depth=4, axis="x"),
        sources=[("plane", {"axis": 0, "index": 5}, 25000.0, 1.0)],
        probes=[("p0", (18, 10, 8)), ("p1", (5, 0, 0))],
        steps=120, store_fields=True,
    ),
    "plane_yz_geom": dict(
        shape=(20, 18, 22), res=2e-3, courant=0.9, pml=dict(depth=2, axis=("y", "z")),
        geometry=dict(kind="blocks", seed=11, n_boxes=3, n_spheres=2),
        sources=[("plane", {"axis": 1, "index": 7}, 12000.0, 1.0),
                 ("plane", {"axis": 2, "index": 20}, 8000.0, 0.5),
                 ("point", (10, 9, 11), 9000.0, 1.0)],
        probes=[("q", (12, 3, 4))],
        steps=100, store_fields=True,
    ),
    "impulse_default_coeffs": dict(
        # reference defaults: rho 1.2, courant 0.95, no PML; impulse written
        # straight into solver.p as tests/test_native_extension.py:247-249 does
        shape=(20, 20, 20), res=2e-3, courant=None, rho=None, pml=None,
        impulse=((10, 10, 10), 1.0), sources=[], probes=[("c", (10, 10, 10))],
        steps=60, store_fields=True,
    ),
    "meters_positions": dict(
        shape=(30, 26, 22), res=1e-3, courant=0.5, pml=dict(depth=5),
        sources=[("point", (0.012, 0.0133, 0.009), 18000.0, 1.0)],
        probes=[("m", (0.02, 0.011, 0.0151))],
        steps=90, store_fields=True,
    ),
    "sdf_geometry": dict(
        shape=(36, 30, 40), res=1e-3, courant=0.5, pml=dict(depth=4),
        geometry=dict(kind="sdf", which="small_enclosure"),
        sources=[("point", (18, 15, 20), 20000.0, 1.0)],
        probes=[("in", (18, 15, 14)), ("out", (5, 5, 5))],
        steps=160, store_fields=True,
    ),
    "mics_geom": dict(
        # omni microphones (trilinear, native batch path) beside probes
        shape=(28, 24, 30), res=1e-3, courant=0.5, pml=dict(depth=4),
        geometry=dict(kind="blocks", seed=21, n_boxes=1, n_spheres=1),
        sources=[("point", (8, 12, 15), 20000.0, 1.0)],
        probes=[("pr", (20, 12, 15))],
        mics=[("m0", (0.0153, 0.0121, 0.0107)), ("m1", (0.0201, 0.0042, 0.0255)),
              ("m2", (0.004, 0.0195, 0.0149)), ("m3", (0.0222, 0.0133, 0.0178))],
        steps=140, store_fields=True,
    ),
    "mics_directional": dict(
        # directional microphones (the reference's Python recording path for
        # every microphone): omni, cardioid, figure-8, supercardioid on an
        # oblique axis, a custom gain(theta); positions at the low and high
        # clamps of the staggered velocity interpolation
        shape=(26, 22, 30), res=1e-3, courant=0.5, pml=dict(depth=4),
        geometry=dict(kind="blocks", seed=33, n_boxes=1, n_spheres=1),
        sources=[("point", (9, 11, 15), 18000.0, 1.0)],
        probes=[("pr", (18, 11, 15))],
        mics=[("om", (0.0153, 0.0121, 0.0107)),
              ("card", (0.0131, 0.0072, 0.0146), dict(pattern="cardioid", direction=(1, 0, 0))),
              ("fig8", (0.0124, 0.0143, 0.0181), dict(pattern="figure8", direction=(0, 1, 0),
                                                      up=(1, 0, 0))),
              ("super", (0.0003, 0.0209996, 0.0066),
               dict(pattern="supercardioid", direction=(0.3, -0.5, 0.8))),
              ("hyper", (0.0247, 0.0004, 0.0288), dict(pattern="hypercardioid",
                                                       direction=(-1, 0.2, 0.1))),
              ("custom", (0.0171, 0.0113, 0.0139), dict(pattern="gain_07_03",
                                                        direction=(0, 0.6, 0.8)))],
        steps=120, store_fields=True,
    ),
    "nu_stretch_blocks": dict(
        # nonuniform grid, geometric growth from the centre (x, z) and from
        # the low end (y, second case); nz % 4 != 0 (scalar warp tiles)
        shape=(30, 26, 34), res=None, courant=0.5, pml=dict(depth=4),
        grid=dict(kind="stretch", base=1e-3, stretch=(1.04, 1.0, 1.06)),
        geometry=dict(kind="blocks", seed=41, n_boxes=1, n_spheres=1),
        sources=[("point", (15, 13, 17), 20000.0, 1.0),
                 ("plane", {"axis": 1, "index": 5}, 12000.0, 0.4)],
        probes=[("a", (8, 13, 17)), ("b", (25, 20, 30))],
        steps=120, store_fields=True,
    ),
    "nu_stretch_low_end": dict(
        shape=(24, 28, 20), res=None, courant=0.6, pml=dict(depth=3, axis=("x", "z")),
        grid=dict(kind="stretch", base=1e-3, stretch=(1.0, 1.05, 1.03), center_fine=False),
        sources=[("point", (6, 9, 10), 25000.0, 1.0)],
        probes=[("a", (18, 20, 10))],
        steps=100, store_fields=True,
    ),
    "nu_regions_sdf": dict(
        # piecewise resolution, SDF geometry voxelised at the grid's own cell
        # centres; nz % 4 == 0 (float4 warp tiles)
        shape=None, res=None, courant=0.5, pml=dict(depth=4),
        grid=dict(kind="regions", x=[(0.0, 0.01, 1e-3), (0.01, 0.03, 5e-4), (0.03, 0.04, 1e-3)],
                  y=[(0.0, 0.024, 1e-3)], z=[(0.0, 0.012, 1.5e-3), (0.012, 0.03, 7.5e-4)]),
        geometry=dict(kind="sdf", which="nu_block"),
        sources=[("point", (30, 12, 16), 20000.0, 1.0)],
        probes=[("a", (12, 12, 16)), ("b", (50, 6, 28))],
        steps=120, store_fields=True,
    ),
    "abc_all_sources": dict(
        # Mur ABC on every axis instead of a PML; sources on boundary planes
        # (injected after the boundary update, as the reference's step does)
        shape=(26, 22, 30), res=1e-3, courant=0.5,
        plane_bcs=[("abc", {})],
        geometry=dict(kind="blocks", seed=52, n_boxes=1, n_spheres=1),
        sources=[("point", (0, 11, 15), 20000.0, 1.0), ("point", (13, 11, 15), 15000.0, 0.5),
                 ("plane", {"axis": 2, "index": 0}, 9000.0, 0.2)],
        probes=[("edge", (0, 11, 15)), ("mid", (13, 5, 20)), ("corner", (25, 21, 29))],
        steps=140, store_fields=True,
    ),
    "rad_pml_mix": dict(
        # a PML on y, radiation impedance at both x ends (constant and
        # pipe-radius reflection), Mur ABC on z, in that order
        shape=(40, 20, 24), res=1e-3, courant=0.5, pml=dict(depth=3, axis="y"),
        plane_bcs=[("rad", {"axis": "x", "side": "high", "reflection_coeff": 0.6}),
                   ("rad", {"axis": "x", "side": "low", "pipe_radius": 0.01}),
                   ("abc", {"axis": "z"})],
        sources=[("point", (8, 10, 12), 18000.0, 1.0)],
        probes=[("hi", (39, 10, 12)), ("lo", (0, 10, 12)), ("zl", (20, 10, 0))],
        steps=160, store_fields=True,
    ),
    "membranes": dict(
        # membrane sources: a circular (0,1) disc on a z plane, a circular
        # (1,1) disc injecting normal velocity on an x plane, a rectangular
        # (1,2) panel on a y plane, and a point source overlapping the disc
        # (source order), with solids cutting into the membranes
        shape=(36, 32, 40), res=1e-3, courant=0.5, pml=dict(depth=4),
        geometry=dict(kind="blocks", seed=61, n_boxes=2, n_spheres=1),
        sources=[("circle", dict(center=(0.018, 0.016, 0.0085), normal_axis="z",
                                 radius=0.007, mode=(0, 1)), 8000.0, 1.0),
                 ("point", (18, 16, 8), 11000.0, 0.5),
                 ("circle", dict(center=(0.0253, 0.015, 0.021), normal_axis="x", radius=0.006,
                                 mode=(1, 1), injection_type="velocity"), 9000.0, 0.002),
                 ("rect", dict(center=(0.017, 0.0245, 0.02), normal_axis="y",
                               size=(0.012, 0.009), mode=(1, 2)), 12000.0, 0.7)],
        probes=[("a", (18, 16, 20)), ("b", (10, 8, 30))],
        steps=120, store_fields=True,
    ),
    "c1_full": dict(
        # the reference quick start, 100^3 x 1000 steps (hashes + traces only)
        shape=(100, 100, 100), res=1e-3, courant=0.5, pml=dict(depth=10),
        sources=[("point", (50, 50, 50), 1000.0, 1.0)],
        probes=[("output", (75, 50, 50))],
        steps=1000, store_fields=False,
    ),
    "served_helmholtz": dict(
        # one request of the served stream's Helmholtz kind: a solid block on
        # the low-x side carved with 9 box-cavity resonators (cavity 10
        # cells, neck radius 3 cells, necks opening to +x), PML 6, the source
        # in front of the necks
        shape=(60, 52, 56), res=1e-3, courant=0.5, pml=dict(depth=6),
        geometry=dict(kind="sdf", which="served_helmholtz"),
        sources=[("point", (28, 26, 28), 2500.0, 1.0)],
        probes=[("near", (28, 26, 28)), ("far", (51, 43, 47))],
        steps=300, store_fields=False,
    ),
    "c2_enclosure_20": dict(
        # the 400^3 enclosure workload, first 20 steps (hashes + traces only)
        shape=(400, 400, 400), res=1e-3, courant=0.5, pml=dict(depth=16),
        geometry=dict(kind="sdf", which="c2_enclosure"),
        sources=[("point", (200, 200, 200), 2000.0, 1.0)],
        probes="c2", steps=20, store_fields=False, big=True,
    ),
}

# --------------------------------------------------------------------------
# ADE path.  The reference's native step never runs the ADE kernels, so the
# golden is the reference's own ADE kernels called in the order of
# _step_python_uniform (core/solver.py:2135-2193).
# pole tuple: ("debye", target, delta_chi, tau) | ("lorentz", target, delta_chi, omega_0, gamma)
ADE_CASES = {
    "debye_2pole": dict(
        shape=(24, 24, 24), res=1e-3, courant=0.5, pml=dict(depth=4),
        materials=[dict(id=1, name="m1", rho=1.204, c=343.0,
                        poles=[("debye", "density", 0.3, 2e-4), ("debye", "modulus", 0.5, 5e-4)],
                        box=((6, 18), (5, 17), (8, 20)))],
        sources=[("point", (12, 12, 3), 20000.0, 1.0)],
        probes=[("in", (12, 12, 12)), ("after", (12, 12, 21))],
        steps=150, store_fields=True,
    ),
    "lorentz_mixed_geom": dict(
        shape=(22, 20, 26), res=1e-3, courant=0.5, pml=dict(depth=3),
        geometry=dict(kind="blocks", seed=5, n_boxes=1, n_spheres=1),
        materials=[
            dict(id=1, name="m1", rho=1.5, c=300.0,
                 poles=[("lorentz", "density", 0.2, 2 * np.pi * 8000.0, 3000.0),
                        ("debye", "modulus", 0.4, 1e-4)],
                 box=((3, 12), (2, 10), (4, 15))),
            dict(id=3, name="m3", rho=1.1, c=360.0,
                 poles=[("lorentz", "modulus", 0.3, 2 * np.pi * 12000.0, 5000.0),
                        ("debye", "density", 0.25, 3e-4)],
                 box=((12, 20), (8, 18), (12, 24))),
        ],
        sources=[("point", (11, 10, 2), 25000.0, 1.0)],
        probes=[("x", (8, 6, 10)), ("y", (16, 13, 18))],
        steps=120, store_fields=True,
    ),
    "split_boxes_geom": dict(
        # material boxes small against the grid, with solids: the GPU splits
        # each step between a warp-tile kernel and the per-cell ADE kernel
        shape=(70, 45, 76), res=1e-3, courant=0.5, pml=dict(depth=5),
        geometry=dict(kind="blocks", seed=8, n_boxes=2, n_spheres=1),
        materials=[
            dict(id=2, name="m2", rho=1.3, c=330.0,
                 poles=[("debye", "density", 0.35, 3e-4), ("debye", "modulus", 0.3, 4e-4)],
                 box=((29, 41), (13, 27), (33, 47))),
            dict(id=5, name="m5", rho=1.1, c=355.0,
                 poles=[("lorentz", "density", 0.15, 2 * np.pi * 9000.0, 4000.0)],
                 box=((40, 47), (20, 31), (45, 52))),
        ],
        sources=[("point", (20, 22, 38), 15000.0, 1.0), ("point", (50, 30, 60), 11000.0, 0.6)],
        probes=[("mid", (35, 20, 40)), ("far", (60, 35, 20))],
        steps=140, store_fields=False,
    ),
    "served_box_debye": dict(
        # one request of the served stream's sealed-box kind with its Debye
        # region: 3-cell walls around a cavity holding the source, a 2-pole
        # Debye block inside the cavity, PML 5
        shape=(50, 44, 48), res=1e-3, courant=0.5, pml=dict(depth=5),
        geometry=dict(kind="sdf", which="served_box"),
        materials=[dict(id=1, name="debye2", rho=1.204, c=343.0,
                        poles=[("debye", "density", 0.4, 3e-4), ("debye", "modulus", 0.6, 5e-4)],
                        box=((26, 34), (15, 25), (20, 30)))],
        sources=[("point", (25, 22, 24), 2000.0, 1.0)],
        probes=[("near", (25, 22, 24)), ("cavity", (30, 28, 30))],
        steps=300, store_fields=False,
    ),
    "materialized_sdf": dict(
        # MaterializedGeometry (geometry/material_assignment.py:48-171): air is
        # the inside of an SDF (a box with a solid sphere taken out, rigid
        # margins outside it), three SDF regions assigned in order -- a sphere,
        # an x cylinder overlapping it (later wins), a box reaching into the
        # rigid margin and the solid sphere (ids only in air)
        shape=(40, 36, 44), res=1e-3, courant=0.5, pml=dict(depth=4),
        materialized=dict(which="mat_air", regions=[
            ("mat_sphere", dict(name="absorber", rho=1.3, c=330.0,
                                poles=[("debye", "density", 0.3, 2e-4),
                                       ("debye", "modulus", 0.4, 4e-4)])),
            ("mat_cylinder", dict(name="resonant", rho=1.1, c=355.0,
                                  poles=[("lorentz", "density", 0.2, 2 * np.pi * 9000.0, 4000.0),
                                         ("debye", "modulus", 0.25, 3e-4)])),
            ("mat_slab", dict(name="slab", rho=1.25, c=340.0,
                              poles=[("debye", "density", 0.35, 5e-4)])),
        ]),
        sources=[("point", (20, 18, 8), 20000.0, 1.0)],
        probes=[("sphere", (24, 18, 20)), ("cyl", (12, 22, 16)), ("slab", (6, 10, 36)),
                ("air", (30, 28, 34))],
        steps=110, store_fields=True,
    ),
    "nu_mixed_geom": dict(
        # ADE on a stretched grid: nonuniform updates and divergence, the
        # corrections with the minimum spacing (core/solver.py:2195-2283)
        shape=(36, 30, 40), res=1e-3, courant=0.5, pml=dict(depth=4),
        grid=dict(kind="stretch", base=1e-3, stretch=(1.03, 1.0, 1.04), center_fine=True),
        geometry=dict(kind="blocks", seed=13, n_boxes=1, n_spheres=1),
        materials=[
            dict(id=1, name="m1", rho=1.4, c=320.0,
                 poles=[("debye", "density", 0.3, 2e-4),
                        ("lorentz", "modulus", 0.25, 2 * np.pi * 9000.0, 4000.0)],
                 box=((8, 20), (6, 18), (10, 24))),
            dict(id=4, name="m4", rho=1.1, c=360.0,
                 poles=[("lorentz", "density", 0.2, 2 * np.pi * 11000.0, 5000.0),
                        ("debye", "modulus", 0.35, 3e-4)],
                 box=((19, 30), (14, 26), (20, 34))),
        ],
        sources=[("point", (18, 15, 3), 20000.0, 1.0),
                 ("plane", {"axis": 1, "index": 4}, 12000.0, 0.2)],
        probes=[("a", (14, 12, 16)), ("b", (24, 20, 28)), ("c", (30, 8, 36))],
        steps=120, store_fields=True,
    ),
}

# --------------------------------------------------------------------------
# Voxelisation: SDFPrimitive.voxelize (geometry/sdf.py:99-125), masks stored
# bit-packed.  (name, grid shape, resolution, tree builder name)
VOXEL_CASES = {
    "box": ((32, 40, 24), 1e-3, "box"),
    "sphere": ((30, 30, 30), 1e-3, "sphere"),
    "cyl_axes": ((40, 36, 32), 1e-3, "cyl_axes"),
    "cyl_oblique": ((32, 32, 32), 1e-3, "cyl_oblique"),
    "csg_mix": ((48, 40, 44), 1e-3, "csg_mix"),
    "translate_scale": ((40, 40, 40), 1e-3, "translate_scale"),
    "rotated": ((44, 40, 48), 1e-3, "rotated"),
    "helmholtz": ((60, 48, 56), 1e-3, "helmholtz"),
    "small_enclosure": ((36, 30, 40), 1e-3, "small_enclosure"),
    "c2_enclosure_4mm": ((100, 100, 100), 4e-3, "c2_enclosure"),
    "cone_smooth": ((48, 44, 40), 1e-3, "cone_smooth"),
    "horns": ((56, 52, 48), 1e-3, "horns"),
    "horn_oblique": ((40, 40, 40), 1e-3, "horn_oblique"),
    "spiral_horn": ((60, 60, 26), 1e-3, "spiral_horn"),
    "helical_tube": ((50, 50, 34), 1e-3, "helical_tube"),
    "bookshelf": ((52, 64, 90), 4e-3, "bookshelf"),
    "cabinet": ((62, 72, 126), 4e-3, "cabinet"),
}
# masks whose reference evaluation rounds through BLAS (np.dot, matmul) or
# NumPy's transcendental functions, or whose host-side constants come from
# those functions on the machine that runs them: cells within that rounding
# of a surface may differ
VOXEL_ROUNDING_CASES = ("cyl_oblique", "rotated", "cone_smooth", "horns", "horn_oblique",
                        "spiral_horn", "helical_tube", "cabinet")


def loudspeaker_cabinet(api, waveform=None):
    """A cabinet with drivers on three faces (one recessed), a divider with
    holes, a diagonal brace, a flared port, an absorber region and a
    Helmholtz array (geometry/loudspeaker.py:52-654)."""
    enc = api.LoudspeakerEnclosure(external_size=(0.24, 0.28, 0.5), wall_thickness=0.018)
    enc.add_driver((0.12, 0.36), 0.13, mounting_depth=0.01, name="woofer", waveform=waveform)
    enc.add_driver((0.12, 0.14), 0.05, baffle_face="top", waveform=waveform, mode=(1, 1))
    enc.add_driver((0.14, 0.42), 0.04, baffle_face="left")
    enc.add_port((0.14, 0.1), 0.04, 0.12, baffle_face="right", flare_ratio=1.5,
                 flare_length=0.03)
    enc.add_chamber_divider(z_position=0.26, thickness=0.016,
                            hole_positions=[(0.06, 0.08, 0.03), (0.18, 0.2, 0.02)])
    enc.add_brace((0.05, 0.14, 0.05), (0.19, 0.14, 0.2), 0.02, 0.03)
    enc.add_absorber_region(((0.03, 0.2, 0.3), (0.21, 0.26, 0.46)), material_id=2)
    enc.add_helmholtz_array(((0.03, 0.03, 0.03), (0.2, 0.24, 0.22)), (300.0, 1200.0), 4)
    return enc


def sdf_tree(api, which):
    """Build a named SDF tree from the API's SDF classes."""
    Box, Sphere, Cylinder = api.Box, api.Sphere, api.Cylinder
    Union, Intersection, Difference = api.Union, api.Intersection, api.Difference
    if which == "box":
        return Box(center=(0.016, 0.0205, 0.0117), size=(0.0101, 0.0203, 0.0071))
    if which == "nu_block":  # a block and a sphere straddling the resolution changes
        return Union(Box(center=(0.0095, 0.0121, 0.0147), size=(0.0043, 0.0102, 0.0061)),
                     Sphere(center=(0.0318, 0.0127, 0.0219), radius=0.0041))
    if which == "sphere":
        return Sphere(center=(0.0151, 0.0149, 0.0153), radius=0.0097)
    if which == "cyl_axes":
        return Union(
            Cylinder(p1=(0.005, 0.018, 0.016), p2=(0.035, 0.018, 0.016), radius=0.0041),
            Cylinder(p1=(0.02, 0.003, 0.0105), p2=(0.02, 0.033, 0.0105), radius=0.0035),
            Cylinder(p1=(0.0295, 0.0095, 0.002), p2=(0.0295, 0.0095, 0.03), radius=0.0050),
        )
    if which == "cyl_oblique":
        return Cylinder(p1=(0.004, 0.006, 0.005), p2=(0.027, 0.025, 0.028), radius=0.0045)
    if which == "csg_mix":
        a = Box(center=(0.024, 0.02, 0.022), size=(0.03, 0.024, 0.028))
        b = Sphere(center=(0.024, 0.02, 0.022), radius=0.016)
        c = Cylinder(p1=(0.024, 0.02, 0.0), p2=(0.024, 0.02, 0.044), radius=0.005)
        d = Box(min_corner=(0.002, 0.002, 0.002), max_corner=(0.01, 0.012, 0.042))
        return Union(Difference(Intersection(a, b), c), d)
    if which == "rotated":  # Rotate (geometry/sdf.py:1303-1390): z, x and oblique axes
        b = Box(center=(0.0, 0.0, 0.0), size=(0.018, 0.008, 0.012)).rotate_z(0.5).translate(
            (0.02, 0.021, 0.019))
        c = Cylinder(p1=(-0.008, 0.0, 0.0), p2=(0.008, 0.0, 0.0), radius=0.004).rotate(
            (1.0, 1.0, 1.0), 0.9).translate((0.024, 0.018, 0.03))
        e = Box(center=(0.0, 0.0, 0.0), size=(0.03, 0.004, 0.006)).rotate_x(-0.35).translate(
            (0.022, 0.03, 0.012))
        return Difference(Union(b, c, e), Sphere(center=(0.02, 0.021, 0.019), radius=0.003))
    if which == "translate_scale":
        s = Sphere(center=(0.0, 0.0, 0.0), radius=0.006).translate((0.02, 0.021, 0.019))
        b = Box(center=(0.0, 0.0, 0.0), size=(0.01, 0.006, 0.008)).scale(1.5).translate(
            (0.012, 0.028, 0.03))
        return Union(s, b)
    if which == "helmholtz":
        H = api.HelmholtzResonator
        return Union(
            H(position=(0.015, 0.012, 0.015), cavity_shape="box", cavity_size=(0.016, 0.014, 0.012),
              neck_length=0.008, neck_radius=0.003, neck_direction=(0, 0, 1)),
            H(position=(0.042, 0.014, 0.02), cavity_shape="sphere", cavity_size=(0.008,),
              neck_length=0.007, neck_radius=0.0035, neck_direction=(0, 1, 0)),
            H(position=(0.03, 0.034, 0.036), cavity_shape="cylinder", cavity_size=(0.007, 0.014),
              neck_length=0.006, neck_radius=0.004, neck_direction=(1, 0, 0)),
        )
    if which == "small_enclosure":
        outer = Box(center=(0.018, 0.015, 0.02), size=(0.024, 0.018, 0.03))
        inner = Box(center=(0.018, 0.015, 0.02), size=(0.018, 0.012, 0.024))
        port = Cylinder(p1=(0.018, 0.015, 0.005), p2=(0.018, 0.015, 0.013), radius=0.0035)
        return Difference(outer, inner, port)
    if which == "c2_enclosure":
        return c2_solid(api)
    if which == "cone_smooth":  # Cone (sdf.py:436-541) and the smooth CSG blends (:736-934)
        frustum = api.Cone(p1=(0.012, 0.022, 0.004), p2=(0.012, 0.022, 0.034), r1=0.008, r2=0.003)
        spike = api.Cone(p1=(0.004, 0.036, 0.03), p2=(0.03, 0.036, 0.03), r1=0.0, r2=0.005)
        blend = api.SmoothUnion(Sphere(center=(0.032, 0.014, 0.012), radius=0.0065),
                                Box(center=(0.038, 0.014, 0.02), size=(0.008, 0.01, 0.012)),
                                0.003)
        lens = api.SmoothIntersection(Sphere(center=(0.033, 0.03, 0.024), radius=0.009),
                                      Sphere(center=(0.039, 0.03, 0.024), radius=0.009), 0.002)
        # the reference's smooth difference is negative wherever the subtracted
        # shape is far away (its blend tends to the minimum of base and the
        # negated shape), so it is bounded by a box here
        bite = Intersection(
            api.SmoothDifference(Box(center=(0.024, 0.01, 0.03), size=(0.014, 0.012, 0.012)),
                                 Sphere(center=(0.03, 0.006, 0.034), radius=0.005), 0.0025),
            Box(center=(0.024, 0.01, 0.03), size=(0.02, 0.016, 0.018)))
        return Union(frustum, spike, blend, lens, bite)
    if which == "horns":  # Horn (sdf.py:937-1148), every flare along a coordinate axis
        return Union(
            api.Horn((0.012, 0.012, 0.004), (0.012, 0.012, 0.04), 0.003, 0.009, "conical"),
            api.Horn((0.04, 0.012, 0.044), (0.04, 0.012, 0.006), 0.0025, 0.01, "exponential"),
            api.Horn((0.004, 0.036, 0.014), (0.05, 0.036, 0.014), 0.003, 0.009, "hyperbolic"),
            api.Horn((0.036, 0.004, 0.034), (0.036, 0.048, 0.034), 0.0025, 0.008, "tractrix"))
    if which == "horn_oblique":
        return api.Horn((0.006, 0.008, 0.007), (0.032, 0.03, 0.033), 0.003, 0.009, "exponential")
    if which == "spiral_horn":  # SpiralHorn (sdf.py:1392-1576), extruded from z = 0
        return api.SpiralHorn(center=(0.03, 0.03), throat_radius=0.003, mouth_radius=0.006,
                              inner_spiral_radius=0.008, outer_spiral_radius=0.022, turns=1.5,
                              height=0.02, profile="exponential")
    if which == "bookshelf":  # geometry/loudspeaker.py:703-742
        return api.bookshelf_speaker(0.2, 0.25, 0.35, 0.13, 0.025).build()
    if which == "cabinet":  # LoudspeakerEnclosure with every kind of part
        return loudspeaker_cabinet(api).build()
    if which == "helical_tube":  # HelicalTube (sdf.py:1579-1721)
        return api.HelicalTube(center=(0.025, 0.025, 0.004), helix_radius=0.013,
                               tube_radius_start=0.003, tube_radius_end=0.005, pitch=0.012,
                               turns=2.0)
    if which == "served_helmholtz":  # as workloads.served_stream builds its Helmholtz kind
        res, lo, hi, cav, neck_r, per = 1e-3, 8, (52, 44, 48), 10, 3, 3
        span = [h - lo for h in hi]
        bx = lo + cav + 6
        rs = []
        for q in range(9):
            a, b = q % per, q // per
            cy = lo + (a + 0.5) * span[1] / per
            cz = lo + (b + 0.5) * span[2] / per
            rs.append(api.HelmholtzResonator(
                position=(lo * res + cav * res / 2 + 2 * res, cy * res, cz * res),
                cavity_shape="box", cavity_size=(cav * res,) * 3, neck_length=4 * res,
                neck_radius=neck_r * res, neck_direction=(1, 0, 0)))
        block = Box(min_corner=(lo * res, lo * res, lo * res),
                    max_corner=(bx * res, hi[1] * res, hi[2] * res))
        return Difference(block, Union(*rs))
    if which == "served_box":  # the served stream's sealed box: 3-cell walls
        res, src, half = 1e-3, (25, 22, 24), (12, 10, 11)
        ctr = [(c + 0.5) * res for c in src]
        return Difference(Box(center=ctr, size=[2 * (h + 3) * res for h in half]),
                          Box(center=ctr, size=[2 * h * res for h in half]))
    if which == "mat_air":  # air volume: a box 2 cells in from the faces, minus a sphere
        return Difference(Box(center=(0.02, 0.018, 0.022), size=(0.036, 0.032, 0.040)),
                          Sphere(center=(0.012, 0.02, 0.03), radius=0.004))
    if which == "mat_sphere":
        return Sphere(center=(0.0245, 0.0185, 0.0205), radius=0.009)
    if which == "mat_cylinder":
        return Cylinder(p1=(0.008, 0.0225, 0.0165), p2=(0.034, 0.0225, 0.0165), radius=0.006)
    if which == "mat_slab":
        return Box(min_corner=(0.0, 0.0, 0.03), max_corner=(0.013, 0.036, 0.044))
    raise KeyError(which)


def c2_solid(api):
    """The enclosure of the 400^3 workload: a 200 x 120 x 300 mm box with
    12 mm walls centred at (0.2, 0.2, 0.2) m, and a radius-25 mm port through
    the z-min wall at its face centre, 80 mm long from the outer face inward."""
    centre = (0.2, 0.2, 0.2)
    outer = api.Box(center=centre, size=(0.2, 0.12, 0.3))
    inner = api.Box(center=centre, size=(0.176, 0.096, 0.276))
    z0 = 0.2 - 0.15
    port = api.Cylinder(p1=(0.2, 0.2, z0), p2=(0.2, 0.2, z0 + 0.08), radius=0.025)
    return api.Difference(outer, inner, port)


def c2_probes(geometry, pml_depth=16, n=8, seed=0):
    """8 seeded uniform-random air cells outside the enclosure walls and
    outside the PML (cells outside the outer box's bounding cells)."""
    rng = np.random.default_rng(seed)
    n_cells = geometry.shape[0]
    lo_box = np.array([100, 140, 50]) - 1   # outer box spans 0.1..0.3, 0.14..0.26, 0.05..0.35 m
    hi_box = np.array([300, 260, 350]) + 1
    out = []
    while len(out) < n:
        c = rng.integers(pml_depth, n_cells - pml_depth, size=3)
        inside_bb = np.all(c >= lo_box) and np.all(c < hi_box)
        if inside_bb or not geometry[tuple(c)]:
            continue
        out.append(tuple(int(v) for v in c))
    return [(f"probe{q}", pos) for q, pos in enumerate(out)]


def _material(api, m):
    """SimpleMaterial from a case's material dict (rho, c, pole tuples)."""
    poles = []
    for pd in m["poles"]:
        if pd[0] == "debye":
            poles.append(api.Pole(pole_type=api.PoleType.DEBYE, delta_chi=pd[2],
                                  target=pd[1], tau=pd[3]))
        else:
            poles.append(api.Pole(pole_type=api.PoleType.LORENTZ, delta_chi=pd[2],
                                  target=pd[1], omega_0=pd[3], gamma=pd[4]))
    return api.SimpleMaterial(name=m["name"], _rho=m["rho"], _c=m["c"], _poles=poles)


def build_case(api, case, ade=False):
    """Construct a solver for ``case`` through the reference-shaped ``api``."""
    g = case.get("grid")
    if g is None:
        grid = api.UniformGrid(shape=case["shape"], resolution=case["res"])
    elif g["kind"] == "stretch":
        grid = api.NonuniformGrid.from_stretch(case["shape"], g["base"], *g["stretch"],
                                               center_fine=g.get("center_fine", True))
    else:
        grid = api.NonuniformGrid.from_regions(g["x"], g["y"], g["z"])
    kw = dict(grid=grid, c=AIR["c"], backend="native")
    rho = case.get("rho", AIR["rho"])
    if rho is not None:          # None: the reference default (1.2)
        kw["rho"] = rho
    if case.get("courant") is not None:
        kw["courant"] = case["courant"]
    solver = api.FDTDSolver(**kw)
    if case.get("pml"):
        solver.add_boundary(api.PML(**case["pml"]))
    for kind, opts in case.get("plane_bcs", []):
        cls = api.ABCFirstOrder if kind == "abc" else api.RadiationImpedance
        solver.add_boundary(cls(**opts))
    geo = case.get("geometry")
    if geo:
        if geo["kind"] == "blocks":
            solver.set_geometry(_mask_blocks(case["shape"], geo["seed"],
                                             geo.get("n_boxes", 2), geo.get("n_spheres", 1)))
        else:
            solver.set_geometry(~sdf_tree(api, geo["which"]).voxelize(solver.grid))
    mg = case.get("materialized")
    if mg:  # MaterializedGeometry: SDF air volume + ordered SDF material regions
        geo = api.MaterializedGeometry(sdf_tree(api, mg["which"]))
        for which, m in mg["regions"]:
            geo.set_material(sdf_tree(api, which), _material(api, m))
        solver.set_geometry(geo)
    for m in case.get("materials", []):
        mid = solver.register_material(_material(api, m), material_id=m["id"])
        solver.set_material_box(mid, *m["box"])
    for kind, pos, f, a in case.get("sources", []):
        if kind == "point":
            solver.add_source(api.GaussianPulse(position=pos, frequency=f, amplitude=a))
        elif kind == "plane":
            solver.add_source(api.GaussianPulse(position=dict(pos), frequency=f, amplitude=a,
                                                source_type="plane"))
        else:  # membrane: pos = constructor options, the waveform a GaussianPulse
            opts = dict(pos)
            cls = (api.CircularMembraneSource if kind == "circle"
                   else api.RectangularMembraneSource)
            wf = api.GaussianPulse(position=(0, 0, 0), frequency=f, amplitude=a)
            solver.add_source(cls(waveform=wf, **opts))
    probes = case.get("probes", [])
    if probes == "c2":
        probes = c2_probes(solver.geometry)
    for name, pos in probes:
        solver.add_probe(name, pos)
    for mic in case.get("mics", []):
        name, pos = mic[0], mic[1]
        opts = dict(mic[2]) if len(mic) > 2 else {}
        if opts.get("pattern") == "gain_07_03":
            opts["pattern"] = gain_07_03
        solver.add_microphone(position=pos, name=name, **opts)
    if case.get("impulse"):
        pos, val = case["impulse"]
        solver.p[pos] = val
    return solver


def dsp_waveforms(api, D):
    """The processed waveforms the dsp check compares (built the same way
    from either API's classes)."""
    src = api.GaussianPulse(position=(0, 0, 0), frequency=2500.0, amplitude=1.0)
    xo = D.Crossover(frequency=1200.0)
    x3 = D.ThreeWayCrossover(low_freq=400.0, high_freq=4000.0, order=4, type="butterworth")
    eq = D.ParametricEQ()
    for f, g, q, kind in ((150.0, 4.0, 0.7, "lowshelf"), (900.0, -3.0, 2.0, "peaking"),
                          (6000.0, 2.5, 0.05, "highshelf"), (60.0, 0.0, 0.7, "highpass"),
                          (12000.0, 0.0, 1.0, "lowpass")):
        eq.add_band(f, g, q, kind)
    return {"lr_low": xo.lowpass(src), "lr_high": xo.highpass(src),
            "bw_woofer": x3.woofer(src), "bw_mid": x3.midrange(src), "bw_tweeter": x3.tweeter(src),
            "bessel_hp": D.FilteredWaveform(src, "highpass", 800.0, order=3, design="bessel"),
            "delayed": D.DelayedWaveform(xo.highpass(src), delay_seconds=2.5e-4),
            "eq": eq.apply(src),
            "baffle": D.create_baffle_step_compensation(0.25).apply(src)}


def random_sdf_tree(api, rng, depth=3):
    """A seeded random SDF tree over every shape and operator the GPU
    voxeliser takes (for point-evaluation checks against the oracle)."""
    def point():
        return tuple(float(v) for v in rng.uniform(0.008, 0.042, 3))

    def leaf():
        kind = int(rng.integers(0, 5))
        if kind == 0:
            return api.Box(center=point(), size=tuple(float(v) for v in rng.uniform(0.004, 0.02, 3)))
        if kind == 1:
            return api.Sphere(center=point(), radius=float(rng.uniform(0.003, 0.012)))
        if kind == 2:
            return api.Cylinder(p1=point(), p2=point(), radius=float(rng.uniform(0.002, 0.008)))
        if kind == 3:
            return api.Cone(p1=point(), p2=point(), r1=float(rng.uniform(0.0, 0.009)),
                            r2=float(rng.uniform(0.002, 0.009)))
        prof = ("conical", "exponential", "hyperbolic", "tractrix")[int(rng.integers(0, 4))]
        return api.Horn(point(), point(), float(rng.uniform(0.002, 0.004)),
                        float(rng.uniform(0.005, 0.01)), prof)

    def node(d):
        if d == 0 or rng.random() < 0.25:
            return leaf()
        op = int(rng.integers(0, 9))
        a, b = node(d - 1), node(d - 1)
        r = float(rng.uniform(0.001, 0.004))
        if op == 0:
            return api.Union(a, b, node(d - 1))
        if op == 1:
            return api.Intersection(a, b)
        if op == 2:
            return api.Difference(a, b)
        if op == 3:
            return api.SmoothUnion(a, b, r)
        if op == 4:
            return api.SmoothIntersection(a, b, r)
        if op == 5:
            return api.SmoothDifference(a, b, r)
        if op == 6:
            return a.translate(tuple(float(v) for v in rng.uniform(-0.004, 0.004, 3)))
        if op == 7:
            return a.scale(float(rng.uniform(0.8, 1.25)))
        return a.rotate(tuple(float(v) for v in rng.uniform(-1, 1, 3)), float(rng.uniform(-1, 1)))

    return node(depth)


# The legacy (binary + JSON) result files: fixed arrays through every
# exporter option, and a small solve with pressure and velocity snapshots
# exported whole (io/legacy.py).  The same calls run against the reference's
# module (tests/golden/make_golden.py ``legacy``) and this package's.
LEGACY_CASE = dict(
    shape=(22, 18, 26), res=1e-3, courant=0.5, pml=dict(depth=3),
    geometry=dict(kind="blocks", seed=5),
    sources=[("point", (7, 9, 12), 25000.0, 1.0),
             ("plane", {"axis": 2, "index": 20}, 15000.0, 0.5)],
    probes=[("a", (15, 9, 12)), ("b", (4, 3, 20))],
    steps=45, snapshot_interval=10,
)


def _collect(d):
    """{relative path: bytes} of every file under d, with the directory's
    own path written as <dir> inside the JSON files (they record paths)."""
    out = {}
    for root, _, names in os.walk(d):
        for n in sorted(names):
            path = os.path.join(root, n)
            data = open(path, "rb").read()
            if n.endswith(".json"):
                data = data.replace(str(d).encode(), b"<dir>")
            out[os.path.relpath(path, d)] = data
    return out


def _meta(m, d):
    return json.dumps(m).replace(str(d), "<dir>")


def legacy_array_exports(L, d):
    """Every array exporter option on fixed arrays (float16 overflow and
    subnormals, a constant field for uint8, both geometry encodings).
    Returns ({call: metadata JSON}, {file: bytes})."""
    rng = np.random.default_rng(21)
    p = (rng.standard_normal((9, 10, 11)) * 50).astype(np.float32)
    p[0, 0, 0], p[1, 1, 1], p[2, 2, 2] = 7.0e4, 1.0e-6, -3.3e-8
    vel = [rng.standard_normal((9, 10, 11)).astype(np.float32) * 1e-3 for _ in range(3)]
    geom = rng.random((9, 10, 11)) > 0.3
    meta = {}
    for fmt in ("float16", "float32", "uint8"):
        for ds in (1, 2):
            meta[f"snap_{fmt}_{ds}"] = L.export_snapshot(p, os.path.join(d, f"s_{fmt}_{ds}.bin"),
                                                         format=fmt, downsample=ds)
    meta["snap_flat_uint8"] = L.export_snapshot(np.full((4, 5, 6), 2.5, np.float32),
                                                os.path.join(d, "flat.bin"), format="uint8")
    for fmt in ("float16", "float32"):
        for inter in (True, False):
            meta[f"vel_{fmt}_{inter}"] = L.export_velocity_snapshot(
                *vel, os.path.join(d, f"v_{fmt}_{int(inter)}"), format=fmt, downsample=3,
                interleaved=inter)
    meta["geom_bin"] = L.export_geometry(geom, os.path.join(d, "g.bin"))
    meta["geom_json"] = L.export_geometry(geom, os.path.join(d, "g.json"), format="json")
    return {k: _meta(v, d) for k, v in meta.items()}, _collect(d)


def legacy_solve_exports(L, solver, d):
    """A finished solve through export_simulation (defaults; float32 at half
    resolution without velocity), export_probe_data of one probe and
    export_metadata with extra keys.  Returns ({call: metadata JSON},
    {file: bytes})."""
    meta = {"sim": L.export_simulation(solver, d, prefix="run"),
            "sim_alt": L.export_simulation(solver, os.path.join(d, "alt"), prefix="alt",
                                           include_velocity=False, snapshot_format="float32",
                                           snapshot_downsample=2),
            "probe_b": L.export_probe_data(solver, os.path.join(d, "b.json"), probe_names=["b"])}
    L.export_metadata(solver, os.path.join(d, "meta_extra.json"), extra={"run": 3, "tag": "x"})
    return {k: _meta(v, d) for k, v in meta.items()}, _collect(d)
