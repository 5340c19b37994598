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
from .materials import Pole, PoleType, SimpleMaterial
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


def random_debye_material(rng):
    """Two Debye poles: tau log-uniform in [1e-5, 1e-3] s, delta_chi uniform
    in [0.1, 1.0], each pole's target drawn (density or modulus)."""
    poles = []
    for _ in range(2):
        tau = float(np.exp(rng.uniform(np.log(1e-5), np.log(1e-3))))
        chi = float(rng.uniform(0.1, 1.0))
        target = "density" if rng.random() < 0.5 else "modulus"
        poles.append(Pole(PoleType.DEBYE, delta_chi=chi, target=target, tau=tau))
    return SimpleMaterial(name="debye2", _rho=RHO_AIR, _c=C_AIR, _poles=poles)


def material_is_stable(material, n=24, steps=1500):
    """Stability screen for a dispersive material: a unit pressure impulse in
    an n^3 grid filled with the material, stepped on the GPU; the material is
    rejected when |p| ever exceeds 10 (the reference's ADE recursion diverges
    for short relaxation times and large strengths)."""
    s = FDTDSolver(grid=UniformGrid((n, n, n), 1e-3), c=C_AIR, rho=RHO_AIR, courant=0.5)
    mid = s.register_material(material)
    s.set_material_box(mid, (0, n), (0, n), (0, n))
    c = n // 2
    s.p[c, c, c] = 1.0
    s.add_probe("c", (c, c, c))
    s.run_steps(steps)
    peak = max(float(np.nanmax(np.abs(s.get_probe_data()["c"]))), float(np.abs(s.p).max()))
    return bool(np.isfinite(peak) and peak <= 10.0), peak


def _place(rng, n, r, pml):
    lo, hi = pml + r, n - pml - r
    if hi <= lo:
        lo, hi = pml, max(pml + 1, n - pml)
    return int(rng.integers(lo, hi))


def batch_workload(seed=0, n_solves=64, screen=True, pml=8):
    """The heterogeneous batch: n_solves grids with edges log-uniform in
    [64, 256] per axis, 1 mm cells, PML 8, 1-6 rigid spheres or boxes
    (radius / half-edge 5-30 cells) in the non-PML interior, one box of a
    2-pole Debye material, a 1-4 kHz pulse at a random air cell, 2 probes,
    500-3000 steps.  Unstable material draws are redrawn (``screen``).
    Returns (solvers, steps, info)."""
    rng = np.random.default_rng(seed)
    solvers, steps, rejected = [], [], 0
    for _ in range(n_solves):
        shape = tuple(int(round(np.exp(rng.uniform(np.log(64), np.log(256))))) for _ in range(3))
        geom = np.ones(shape, dtype=bool)
        for _ in range(int(rng.integers(1, 7))):
            r = int(rng.integers(5, 31))
            cen = [_place(rng, n, r, pml) for n in shape]
            lo = [max(0, c - r) for c in cen]
            hi = [min(n, c + r + 1) for c, n in zip(cen, shape)]
            if rng.random() < 0.5:  # sphere
                ii, jj, kk = np.ogrid[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
                ball = (ii - cen[0]) ** 2 + (jj - cen[1]) ** 2 + (kk - cen[2]) ** 2 <= r * r
                geom[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] &= ~ball
            else:
                geom[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = False
        s = FDTDSolver(grid=UniformGrid(shape, 1e-3), c=C_AIR, rho=RHO_AIR, courant=0.5)
        s.add_boundary(PML(depth=pml))
        s.set_geometry(geom)
        while True:
            mat = random_debye_material(rng)
            if not screen or material_is_stable(mat)[0]:
                break
            rejected += 1
        mid = s.register_material(mat)
        half = [int(rng.integers(5, 21)) for _ in range(3)]
        cen = [_place(rng, n, h, pml) for n, h in zip(shape, half)]
        s.set_material_box(mid, *[(max(0, c - h), min(n, c + h)) for c, h, n in zip(cen, half, shape)])

        def air_cell():
            while True:
                c = tuple(int(rng.integers(pml, n - pml)) for n in shape)
                if geom[c]:
                    return c

        s.add_source(GaussianPulse(position=air_cell(), frequency=float(rng.uniform(1000, 4000))))
        s.add_probe("p0", air_cell())
        s.add_probe("p1", air_cell())
        solvers.append(s)
        steps.append(int(rng.integers(500, 3001)))
    return solvers, steps, {"rejected_materials": rejected, "seed": seed}


def served_stream(seed=0, n_requests=1000, rate=200.0, edges=(48, 320), steps=(500, 5000),
                  pml=(8, 16), ade_fraction=0.5, screen=True):
    """The request stream: Poisson arrivals (``rate`` per second), grid
    edges log-uniform in ``edges`` per axis, steps uniform in ``steps``, PML
    uniform in ``pml``, geometry drawn from free field / a sealed box / a
    block of 4-32 Helmholtz resonators (neck radius 3-8 cells, cavity 10-20
    cells), an optional 1-2 pole Debye region.  Returns a list of
    server.Request whose ``build`` constructs the solver on admission.

    Every random parameter of a request is drawn here, including its Debye
    material, which is redrawn until it passes the stability screen
    (material_is_stable, on the GPU): the screen is the workload's rejection
    rule, not part of serving, so it runs before the stream starts and
    ``build`` only constructs."""
    from .resonator import HelmholtzResonator
    from .sdf import Union
    from .server import Request, solve_bytes

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        shape = tuple(int(round(np.exp(rng.uniform(np.log(edges[0]), np.log(edges[1])))))
                      for _ in range(3))
        n_steps = int(rng.integers(steps[0], steps[1] + 1))
        depth = int(rng.integers(pml[0], pml[1] + 1))
        kind = ["free", "box", "helmholtz"][int(rng.integers(0, 3))]
        res = 1e-3
        spec = dict(shape=shape, depth=depth, kind=kind, seed=int(rng.integers(0, 2**31)))
        n_poles = 0
        if rng.random() < ade_fraction:
            n_poles = int(rng.integers(1, 3))
        spec["n_poles"] = n_poles
        nbytes = solve_bytes(shape, geometry=kind != "free", debye_poles=n_poles)
        # the request's own draws, in the order they are used
        r = np.random.default_rng(spec["seed"])
        inner_lo = [depth + 2 for _ in shape]
        inner_hi = [n - depth - 2 for n in shape]
        if kind == "helmholtz":
            spec["nres"] = int(r.integers(4, 33))
            spec["cav"] = int(r.integers(10, 21))
            spec["neck_r"] = int(r.integers(3, 9))
        if n_poles:
            while True:
                mat = random_debye_material(r)
                mat._poles = mat._poles[:n_poles]
                if not screen or material_is_stable(mat)[0]:
                    break
            spec["material"] = mat
            half = [int(r.integers(3, 9)) for _ in shape]
            spec["box"] = [(c - h, c + h) for c, h in zip(
                [int(r.integers(lo + h, max(lo + h + 1, hi - h)))
                 for lo, hi, h in zip(inner_lo, inner_hi, half)], half)]
        spec["frequency"] = float(r.uniform(1000, 4000))

        def build(spec=spec, res=res):
            shp, d = spec["shape"], spec["depth"]
            s = FDTDSolver(grid=UniformGrid(shp, res), c=C_AIR, rho=RHO_AIR, courant=0.5)
            s.add_boundary(PML(depth=d))
            inner_lo = [d + 2 for _ in shp]
            inner_hi = [n - d - 2 for n in shp]
            src = tuple((lo + hi) // 2 for lo, hi in zip(inner_lo, inner_hi))
            if spec["kind"] == "box":
                # sealed box: 3-cell walls around a cavity holding the source
                half = [max(4, (hi - lo) // 3) for lo, hi in zip(inner_lo, inner_hi)]
                ctr = [(c + 0.5) * res for c in src]
                outer = Box(center=ctr, size=[2 * (h + 3) * res for h in half])
                cav = Box(center=ctr, size=[2 * h * res for h in half])
                s.set_geometry_sdf(Difference(outer, cav))
            elif spec["kind"] == "helmholtz":
                # a block of resonators on the low-x side, necks opening to +x
                span = [hi - lo for lo, hi in zip(inner_lo, inner_hi)]
                nres, cav, neck_r = spec["nres"], spec["cav"], spec["neck_r"]
                per = max(1, int(np.ceil(np.sqrt(nres))))
                bx = inner_lo[0] + cav + 6
                res_list = []
                for q in range(nres):
                    a, b = q % per, q // per
                    cy = inner_lo[1] + (a + 0.5) * span[1] / per
                    cz = inner_lo[2] + (b + 0.5) * span[2] / per
                    res_list.append(HelmholtzResonator(
                        position=(inner_lo[0] * res + cav * res / 2 + 2 * res, cy * res, cz * res),
                        cavity_shape="box", cavity_size=(cav * res,) * 3, neck_length=4 * res,
                        neck_radius=neck_r * res, neck_direction=(1, 0, 0)))
                block = Box(min_corner=(inner_lo[0] * res, inner_lo[1] * res, inner_lo[2] * res),
                            max_corner=(bx * res, inner_hi[1] * res, inner_hi[2] * res))
                s.set_geometry_sdf(Difference(block, Union(*res_list)))
                src = (min(inner_hi[0] - 1, bx + 4), src[1], src[2])
            if spec["n_poles"]:
                mid = s.register_material(spec["material"])
                s.set_material_box(mid, *spec["box"])
            geom = s.geometry
            if not geom[src]:
                air = np.argwhere(geom[inner_lo[0]:inner_hi[0], inner_lo[1]:inner_hi[1],
                                       inner_lo[2]:inner_hi[2]])
                if len(air):
                    src = tuple(int(v) + lo for v, lo in zip(air[len(air) // 2], inner_lo))
            s.add_source(GaussianPulse(position=src, frequency=spec["frequency"]))
            s.add_probe("near", src)
            s.add_probe("far", tuple(hi - 1 for hi in inner_hi))
            s.precompute_sources(spec["steps"])
            return s

        spec["steps"] = n_steps
        out.append(Request(rid=rid, build=build, steps=n_steps, arrival=t, nbytes=nbytes,
                           cells=int(np.prod(shape))))
    return out


def design_field(shape, region=64, seed=0, sigma=4.0):
    """Seeded smooth density-scale field: uniform noise on a central
    region^3 box, Gaussian-filtered (sigma cells), renormalised to [0, 1];
    zero outside the box."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    theta = np.zeros(shape, dtype=np.float64)
    r = [min(region, n) for n in shape]
    lo = [(n - m) // 2 for n, m in zip(shape, r)]
    box = gaussian_filter(rng.uniform(0.0, 1.0, size=r), sigma=sigma, mode="reflect")
    box = (box - box.min()) / max(box.max() - box.min(), 1e-300)
    theta[lo[0]:lo[0] + r[0], lo[1]:lo[1] + r[1], lo[2]:lo[2] + r[2]] = box
    return theta


def quick_start_100(**kw) -> FDTDSolver:
    s = FDTDSolver(grid=UniformGrid((100, 100, 100), 1e-3), c=C_AIR, rho=RHO_AIR, courant=0.5,
                   backend="native", **kw)
    s.add_boundary(PML(depth=10))
    s.add_source(GaussianPulse(position=(50, 50, 50), frequency=1000.0, amplitude=1.0))
    s.add_probe("output", (75, 50, 50))
    return s
