"""CPU oracle for the strata-fdtd time-step path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs may import this module.  The product package never does.

It restates the reference's solver API (same class names, arguments and step
order; paths relative to src/strata_fdtd/ of rjwalters/strata-fdtd) on top of
``liboracle.so`` (oracle/sf_oracle.c), the C restatement of the reference
native kernels.  ``precision="f32"`` reproduces FDTDSolver(backend="native")
bit for bit (pinned against the reference's own outputs in tests/golden/);
``precision="f64"`` runs the same arithmetic in double to state the error of
an FP32 result.  ADE materials are stepped in the order of
_step_python_uniform / _step_python_nonuniform (core/solver.py:2135-2193,
2195-2283) with the native kernels' arithmetic (the reference's native step
skips ADE altogether); on a nonuniform grid that is the nonuniform velocity
and pressure updates, the uniform-dx velocity and pressure corrections and
compute_divergence_nonuniform, the calls its python path makes when the
native module is loaded (solver.py:3150-3170, 3294-3305).

Voxelisation restates geometry/sdf.py with the same NumPy calls, so on one
machine it reproduces SDFPrimitive.voxelize exactly.
"""
from __future__ import annotations

import ctypes
import enum
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib():
    """Load (building on first use) oracle/_build/liboracle.so."""
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        src = os.path.join(HERE, "sf_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
        _LIB = ctypes.CDLL(path)
        _declare(_LIB)
    return _LIB


def _declare(L):
    P, I, L64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    for suf, R in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
        sig = {
            "update_velocity": [P, P, P, P, I, I, I, R],
            "update_pressure": [P, P, P, P, P, I, I, I, R],
            "update_velocity_nu": [P, P, P, P, I, I, I, R, P, P, P],
            "update_pressure_nu": [P, P, P, P, P, I, I, I, R, P, P, P],
            "apply_rigid": [P, P, P, P, I, I, I],
            "boundary_faces": [P, I, I, I, I, P],
            "pml_decay": [P, I, R, P],
            "pml_velocity": [P, P, P, P, P, P, I, I, I],
            "pml_pressure": [P, P, P, P, I, I, I],
            "inject": [P, P, I, I, I, I, I, I, I, D],
            "ade_debye": [P, P, P, I, R, R, L64],
            "ade_lorentz": [P, P, P, P, I, R, R, R, L64],
            "ade_velocity_correction": [P, P, P, P, P, I, R, I, I, I],
            "ade_pressure_correction": [P, P, P, I, R, L64],
            "divergence": [P, P, P, P, I, I, I, R],
            "divergence_nu": [P, P, P, P, I, I, I, P, P, P],
            "run_plain": [P, P, P, P, P, L64, P, P],
            "omp_threads": [],
            "set_threads": [I],
        }
        for name, args in sig.items():
            fn = getattr(L, f"orc_{name}_{suf}")
            fn.argtypes = args
            fn.restype = L64 if name == "boundary_faces" else (I if name == "omp_threads" else None)


def _ptr(a):
    return None if a is None else a.ctypes.data


class _PlanF(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("cv", ctypes.c_float), ("cp", ctypes.c_float),
                ("geom", ctypes.c_void_p), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("dz", ctypes.c_void_p), ("n_src", ctypes.c_int), ("src", ctypes.c_void_p),
                ("n_probe", ctypes.c_int), ("probe_cell", ctypes.c_void_p)]


class _PlanD(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("cv", ctypes.c_double), ("cp", ctypes.c_double),
                ("geom", ctypes.c_void_p), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("dz", ctypes.c_void_p), ("n_src", ctypes.c_int), ("src", ctypes.c_void_p),
                ("n_probe", ctypes.c_int), ("probe_cell", ctypes.c_void_p)]


def set_threads(n):
    lib().orc_set_threads_f32(int(n))


def threads():
    return int(lib().orc_omp_threads_f32())


# ---------------------------------------------------------------------------
# Grid (core/grid.py:51-146)
class UniformGrid:
    def __init__(self, shape, resolution):
        self.shape = tuple(int(n) for n in shape)
        self.resolution = float(resolution)
        r = self.resolution
        self.x_coords = np.arange(self.shape[0]) * r + r / 2
        self.y_coords = np.arange(self.shape[1]) * r + r / 2
        self.z_coords = np.arange(self.shape[2]) * r + r / 2
        self.min_spacing = r
        self.is_uniform = True


class NonuniformGrid:
    """core/grid.py:148-532: cell centres per axis, spacing (x[i+1]-x[i-1])/2
    inside and the neighbour distance at the ends, from_stretch and
    from_regions coordinate generators, float32 inverse spacings."""

    def __init__(self, x_coords, y_coords, z_coords):
        self.x_coords, self.y_coords, self.z_coords = (
            np.asarray(c, dtype=np.float64).ravel() for c in (x_coords, y_coords, z_coords))
        self.dx, self.dy, self.dz = (self._spacing(c) for c in
                                     (self.x_coords, self.y_coords, self.z_coords))
        self.shape = (len(self.x_coords), len(self.y_coords), len(self.z_coords))
        self.min_spacing = float(min(np.min(self.dx), np.min(self.dy), np.min(self.dz)))
        self.is_uniform = False

    @staticmethod
    def _spacing(c):
        s = np.zeros(len(c), dtype=np.float64)
        for i in range(1, len(c) - 1):
            s[i] = (c[i + 1] - c[i - 1]) / 2
        s[0] = c[1] - c[0]
        s[-1] = c[-1] - c[-2]
        return s

    @classmethod
    def from_stretch(cls, shape, base_resolution, stretch_x=1.0, stretch_y=1.0, stretch_z=1.0,
                     center_fine=True):
        return cls(*(cls._stretched(n, base_resolution, st, center_fine)
                     for n, st in zip(shape, (stretch_x, stretch_y, stretch_z))))

    @staticmethod
    def _stretched(n, b, st, center_fine):
        if st == 1.0:
            return np.arange(n, dtype=np.float64) * b + b / 2
        if not center_fine:
            sizes = b * (st ** np.arange(n, dtype=np.float64))
            return np.cumsum(sizes) - sizes / 2
        h = n // 2
        sizes = b * (st ** np.arange(h, dtype=np.float64))
        pos = np.cumsum(sizes) - sizes[0] / 2
        left = -pos[::-1] - sizes[::-1] / 2
        if n % 2 == 0:
            coords = np.concatenate([left, pos + sizes / 2])
        else:
            right = pos[1:] + sizes[1:] / 2 if h > 0 else np.array([])
            coords = np.concatenate([left, np.array([0.0]), right])
        return coords - coords[0] + b / 2

    @classmethod
    def from_regions(cls, x_regions, y_regions=None, z_regions=None):
        return cls(*(cls._regions(r) for r in (x_regions, y_regions or x_regions,
                                                z_regions or x_regions)))

    @staticmethod
    def _regions(regions):
        out = []
        for start, end, res in regions:
            n = max(1, int(round((end - start) / res)))
            step = (end - start) / n
            rc = start + (np.arange(n) + 0.5) * step
            if out and len(rc) > 0 and abs(rc[0] - out[-1]) < step / 2:
                rc = rc[1:]
            out.extend(rc.tolist())
        return np.array(out, dtype=np.float64)

    def get_spacing_arrays_for_stencil(self):
        f = np.float32
        return {"inv_dx_face": (1.0 / np.diff(self.x_coords)).astype(f),
                "inv_dx_cell": (1.0 / self.dx).astype(f),
                "inv_dy_face": (1.0 / np.diff(self.y_coords)).astype(f),
                "inv_dy_cell": (1.0 / self.dy).astype(f),
                "inv_dz_face": (1.0 / np.diff(self.z_coords)).astype(f),
                "inv_dz_cell": (1.0 / self.dz).astype(f)}


# ---------------------------------------------------------------------------
# Source (core/solver.py:152-207)
@dataclass
class GaussianPulse:
    position: object
    frequency: float
    bandwidth: float | None = None
    amplitude: float = 1.0
    source_type: str = "point"

    def __post_init__(self):
        if self.bandwidth is None:
            self.bandwidth = 2.0 * self.frequency

    def waveform(self, t, dt):
        sigma = 1.0 / (np.pi * self.bandwidth)
        t0 = 4.0 * sigma
        envelope = np.exp(-((t - t0) ** 2) / (2 * sigma**2))
        carrier = np.sin(2 * np.pi * self.frequency * (t - t0))
        return self.amplitude * envelope * carrier


# ---------------------------------------------------------------------------
# Materials (materials/base.py:55-213, 509-545)
class PoleType(enum.Enum):
    DEBYE = "debye"
    LORENTZ = "lorentz"


@dataclass
class Pole:
    pole_type: PoleType
    delta_chi: float
    target: str
    tau: float | None = None
    omega_0: float | None = None
    gamma: float | None = None

    @property
    def is_debye(self):
        return self.pole_type == PoleType.DEBYE

    def fdtd_coefficients(self, dt):
        if self.is_debye:
            tau_dt = self.tau / dt
            denom = 1 + tau_dt
            return (tau_dt / denom, self.delta_chi / denom)
        w0, g = self.omega_0, self.gamma
        dt2 = dt * dt
        c = 1 + g * dt / 2
        a = (2 - w0**2 * dt2) / c
        b = -(1 - g * dt / 2) / c
        d = self.delta_chi * w0**2 * dt2 / c
        return (a, b, d)


@dataclass
class SimpleMaterial:
    name: str
    _rho: float = 1.2
    _c: float = 343.0
    _poles: list = field(default_factory=list)

    @property
    def rho_inf(self):
        return self._rho

    @property
    def K_inf(self):
        return self._rho * self._c**2

    @property
    def poles(self):
        return self._poles


# ---------------------------------------------------------------------------
# PML (boundaries/_boundaries.py:104-377): sigma profile + multiplicative decay
class PML:
    def __init__(self, depth=10, axis="all", max_sigma=None, order=3):
        self.depth = depth
        self.order = order
        self.axes = ("x", "y", "z") if axis == "all" else ((axis,) if isinstance(axis, str) else axis)
        self._max_sigma = max_sigma

    def initialize(self, solver):
        nx, ny, nz = solver.shape
        if self._max_sigma is None:
            R_target = 1e-6
            d = self.depth * solver.grid.min_spacing
            self._max_sigma = -(self.order + 1) * solver.c * np.log(R_target) / (2 * d)
        dtype = np.float64 if solver.precision == "f64" else np.float32
        g = solver.grid
        if g.is_uniform:
            sig = [self._profile(n, dtype) if a in self.axes else None
                   for n, a in zip((nx, ny, nz), ("x", "y", "z"))]
        else:
            sig = [self._profile_nu(c, s, dtype) if a in self.axes else None
                   for c, s, a in zip((g.x_coords, g.y_coords, g.z_coords), (g.dx, g.dy, g.dz),
                                      ("x", "y", "z"))]
        self._sigma_x, self._sigma_y, self._sigma_z = sig
        self.decay = []
        for s in sig:
            if s is None:
                self.decay.append(None)
            elif solver.precision == "f64":
                self.decay.append(np.exp(-s * solver.dt))
            else:  # pml.cpp:13-45, expf in float with dt rounded to float
                out = np.zeros(len(s), dtype=np.float32)
                lib().orc_pml_decay_f32(s.ctypes.data, len(s), float(np.float32(solver.dt)),
                                        out.ctypes.data)
                self.decay.append(out)

    def _profile_nu(self, coords, sp, dtype):
        """_boundaries.py:257-315: physical distance from the PML interface
        over the PML thickness."""
        n = len(coords)
        sigma = np.zeros(n, dtype=dtype)
        d = self.depth if self.depth < n // 2 else max(1, n // 4)
        lt, rt = float(np.sum(sp[:d])), float(np.sum(sp[-d:]))
        li = coords[d] - sp[d] / 2 if d < n else coords[-1]
        ri = coords[n - d - 1] + sp[n - d - 1] / 2 if n - d > 0 else coords[0]
        for i in range(d):
            nd = min(1.0, (li - coords[i]) / lt) if lt > 0 else 0.0
            sigma[i] = self._max_sigma * (nd ** self.order)
        for i in range(n - d, n):
            nd = min(1.0, (coords[i] - ri) / rt) if rt > 0 else 0.0
            sigma[i] = self._max_sigma * (nd ** self.order)
        return sigma

    def _profile(self, n, dtype):
        sigma = np.zeros(n, dtype=dtype)
        d = self.depth
        for i in range(d):
            sigma[i] = self._max_sigma * (((d - i) / d) ** self.order)
        for i in range(n - d, n):
            sigma[i] = self._max_sigma * (((i - (n - d - 1)) / d) ** self.order)
        return sigma


class _Membrane:
    """Membrane sources (solver.py:210-755): mode-shape weights on the grid
    plane nearest the centre, normalised to 1."""

    source_type = "membrane"

    def __init__(self, center, normal_axis, waveform, mode, injection_type="pressure"):
        self.center, self.normal_axis, self.waveform = center, normal_axis, waveform
        self.mode, self.injection_type, self._w = mode, injection_type, None

    def _frame(self, grid):
        X, Y, Z = np.meshgrid(grid.x_coords, grid.y_coords, grid.z_coords, indexing="ij")
        ax = "xyz".index(self.normal_axis)
        comps = [X - self.center[0], Y - self.center[1], Z - self.center[2]]
        a, b = [c for q, c in enumerate(comps) if q != ax]
        coords = (grid.x_coords, grid.y_coords, grid.z_coords)[ax]
        k = int(np.argmin(np.abs(coords - self.center[ax])))
        plane = np.zeros(grid.shape, dtype=bool)
        idx = [slice(None)] * 3
        idx[ax] = k
        plane[tuple(idx)] = True
        return a, b, plane

    def weights(self, grid):
        a, b, plane = self._frame(grid)
        mask = plane & self._inside(a, b)
        w = np.zeros(grid.shape, dtype=np.float64)
        shape = np.abs(np.where(self._inside(a[mask], b[mask]), self._shape(a[mask], b[mask]),
                                0.0))
        mx = np.max(shape)
        w[mask] = shape / mx if mx > 1e-10 else np.zeros_like(shape)
        return w


class CircularMembraneSource(_Membrane):
    _Z = {(0, 1): 2.4048255576957727, (0, 2): 5.5200781102863115, (1, 1): 3.8317059702075125,
          (1, 2): 7.0155866698156190, (2, 1): 5.1356223018406826, (2, 2): 8.4172441403998649}

    def __init__(self, center, normal_axis, waveform, radius, mode=(0, 1),
                 injection_type="pressure"):
        super().__init__(center, normal_axis, waveform, mode, injection_type)
        from scipy.special import jn_zeros
        self.radius = radius
        self.alpha = self._Z.get(tuple(mode)) or jn_zeros(mode[0], mode[1])[-1]

    def _inside(self, a, b):
        return np.sqrt(a**2 + b**2) <= self.radius

    def _shape(self, a, b):
        from scipy.special import j0, jv
        rho = np.sqrt(a**2 + b**2) / self.radius
        m = self.mode[0]
        if m == 0:
            return j0(self.alpha * rho)
        return jv(m, self.alpha * rho) * np.cos(m * np.arctan2(b, a))


class RectangularMembraneSource(_Membrane):
    def __init__(self, center, normal_axis, waveform, size, mode=(1, 1),
                 injection_type="pressure"):
        super().__init__(center, normal_axis, waveform, mode, injection_type)
        self.size = size

    def _inside(self, a, b):
        return (np.abs(a) <= self.size[0] / 2) & (np.abs(b) <= self.size[1] / 2)

    def _shape(self, a, b):
        m, n = self.mode
        return (np.sin(m * np.pi * (a / self.size[0] + 0.5))
                * np.sin(n * np.pi * (b / self.size[1] + 0.5)))


class ABCFirstOrder:
    """_boundaries.py:420-527, the same NumPy operations (the Mur
    coefficient is a NumPy float64, so each plane update runs in FP64 and is
    rounded into the float32 field)."""

    def __init__(self, axis="all"):
        self.axes = ("x", "y", "z") if axis == "all" else ((axis,) if isinstance(axis, str)
                                                           else tuple(axis))

    def initialize(self, solver):
        nx, ny, nz = solver.shape
        self._coeff = (solver.c * solver.dt - solver.dx) / (solver.c * solver.dt + solver.dx)
        z = np.float32
        self.prev = {a: [np.zeros(s, dtype=z), np.zeros(s, dtype=z)]
                     for a, s in (("x", (ny, nz)), ("y", (nx, nz)), ("z", (nx, ny)))
                     if a in self.axes}

    def apply_pressure(self, solver):
        p, c = solver.p, self._coeff
        for a, ax in (("x", 0), ("y", 1), ("z", 2)):
            if a not in self.prev:
                continue
            pm = np.moveaxis(p, ax, 0)  # a view: writes land in p
            lo, hi = self.prev[a]
            pm[0] = lo + c * (pm[1] - pm[0])
            self.prev[a][0] = pm[1].copy()
            pm[-1] = hi + c * (pm[-2] - pm[-1])
            self.prev[a][1] = pm[-2].copy()


class RadiationImpedance:
    """_boundaries.py:529-793 with constant reflection or from a pipe radius."""

    def __init__(self, axis, side, reflection_coeff=None, pipe_radius=None):
        self.axis, self.side = axis, side
        self.R, self.radius = reflection_coeff, pipe_radius

    def initialize(self, solver):
        nx, ny, nz = solver.shape
        if self.R is None:
            ka = (2 * np.pi * 1000 / solver.c) * self.radius
            z = (ka ** 2) / 4
            self.R = min(abs((z - 1) / (z + 1)), 0.95)
        shape = {"x": (ny, nz), "y": (nx, nz), "z": (nx, ny)}[self.axis]
        self.prev = np.zeros(shape, dtype=np.float32)

    def apply_pressure(self, solver):
        p, R = solver.p, self.R
        mur = (solver.c * solver.dt - solver.dx) / (solver.c * solver.dt + solver.dx)
        pm = np.moveaxis(p, "xyz".index(self.axis), 0)
        b, i = (0, 1) if self.side == "low" else (-1, -2)
        abc = self.prev + mur * (pm[i] - pm[b])
        pm[b] = R * pm[i] + (1 - R) * abc
        self.prev[:] = pm[i]


# ---------------------------------------------------------------------------
# SDF (geometry/sdf.py), same NumPy calls as the reference
class SDFPrimitive:
    def voxelize(self, grid):
        X, Y, Z = np.meshgrid(grid.x_coords, grid.y_coords, grid.z_coords, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        return self.sdf(pts).reshape(grid.shape) <= 0

    def translate(self, offset):
        return Translate(self, offset)

    def scale(self, factor):
        return Scale(self, factor)

    def rotate(self, axis, angle):
        return Rotate(self, axis=axis, angle=angle)

    def rotate_x(self, angle):
        return self.rotate((1, 0, 0), angle)

    def rotate_y(self, angle):
        return self.rotate((0, 1, 0), angle)

    def rotate_z(self, angle):
        return self.rotate((0, 0, 1), angle)


class Box(SDFPrimitive):  # sdf.py:232-299
    def __init__(self, center=None, size=None, min_corner=None, max_corner=None):
        if center is not None and size is not None:
            self.center = np.array(center, dtype=np.float64)
            self.size = np.array(size, dtype=np.float64)
        else:
            lo = np.array(min_corner, dtype=np.float64)
            hi = np.array(max_corner, dtype=np.float64)
            self.center = (lo + hi) / 2
            self.size = hi - lo

    def sdf(self, points):
        q = np.abs(np.asarray(points, dtype=np.float64) - self.center) - self.size / 2
        return np.linalg.norm(np.maximum(q, 0), axis=1) + np.minimum(np.max(q, axis=1), 0)


class Sphere(SDFPrimitive):  # sdf.py:302-338
    def __init__(self, center, radius):
        self.center = np.array(center, dtype=np.float64)
        self.radius = float(radius)

    def sdf(self, points):
        return np.linalg.norm(np.asarray(points, dtype=np.float64) - self.center, axis=1) - self.radius


class Cylinder(SDFPrimitive):  # sdf.py:341-433
    def __init__(self, p1, p2, radius):
        self.p1 = np.array(p1, dtype=np.float64)
        self.p2 = np.array(p2, dtype=np.float64)
        self.radius = float(radius)
        self.axis = self.p2 - self.p1
        self.length = np.linalg.norm(self.axis)
        self.axis_normalized = self.axis / self.length

    def sdf(self, points):
        points = np.asarray(points, dtype=np.float64)
        v = points - self.p1
        t = np.dot(v, self.axis_normalized)
        tc = np.clip(t, 0, self.length)
        closest = self.p1 + tc[:, np.newaxis] * self.axis_normalized
        radial = np.linalg.norm(points - closest, axis=1)
        axial = np.maximum(0, np.abs(t - self.length / 2) - self.length / 2)
        inside = (t >= 0) & (t <= self.length)
        return np.where(inside, radial - self.radius,
                        np.sqrt((radial - self.radius) ** 2 + axial**2))


class Cone(SDFPrimitive):  # sdf.py:436-541
    def __init__(self, p1, p2, r1, r2):
        self.p1 = np.array(p1, dtype=np.float64)
        self.p2 = np.array(p2, dtype=np.float64)
        self.r1, self.r2 = float(r1), float(r2)
        axis = self.p2 - self.p1
        self.length = np.linalg.norm(axis)
        self.axis_normalized = axis / self.length

    def sdf(self, points):
        points = np.asarray(points, dtype=np.float64)
        t = np.dot(points - self.p1, self.axis_normalized) / self.length
        tc = np.clip(t, 0, 1)
        rt = self.r1 + tc * (self.r2 - self.r1)
        closest = self.p1 + (tc * self.length)[:, np.newaxis] * self.axis_normalized
        radial = np.linalg.norm(points - closest, axis=1)
        axial = np.maximum(0, np.abs(t - 0.5) - 0.5) * self.length
        inside = (t >= 0) & (t <= 1)
        return np.where(inside, radial - rt, np.sqrt((radial - rt) ** 2 + axial**2))


class Horn(SDFPrimitive):  # sdf.py:937-1148
    def __init__(self, throat_position, mouth_position, throat_radius, mouth_radius,
                 profile="exponential"):
        self.throat = np.array(throat_position, dtype=np.float64)
        mouth = np.array(mouth_position, dtype=np.float64)
        self.r0, r1 = float(throat_radius), float(mouth_radius)
        self.profile = profile
        axis = mouth - self.throat
        self.L = np.linalg.norm(axis)
        self.axis = axis / self.L
        a0, am = np.pi * self.r0**2, np.pi * r1**2
        if profile == "conical":
            self.k = np.sqrt(am / a0) - 1
        elif profile == "exponential":
            self.k = np.log(am / a0) / (2 * self.L)
        elif profile == "hyperbolic":
            self.k = np.arccosh(np.sqrt(am / a0)) / self.L
        else:
            self.k = self.L / np.arccos(np.power(a0 / am, 0.25))

    def sdf(self, points):
        v = np.asarray(points, dtype=np.float64) - self.throat
        t = np.dot(v, self.axis)
        tc = np.clip(t / self.L, 0, 1)
        r = np.linalg.norm(v - np.outer(t, self.axis), axis=1)
        x = tc * self.L
        if self.profile == "conical":
            hr = self.r0 * (1 + self.k * tc)
        elif self.profile == "exponential":
            hr = self.r0 * np.exp(self.k * x)
        elif self.profile == "hyperbolic":
            hr = self.r0 * np.cosh(self.k * x)
        else:
            hr = self.r0 / np.cos(x / self.k) ** 2
        rd = r - hr
        inside = (t >= 0) & (t <= self.L)
        return np.where(inside, rd, np.sqrt(rd**2 + np.maximum(-t, t - self.L) ** 2))


def _polyline_distance(points, path):  # geometry/paths.py:226-294
    best = np.full(points.shape[0], np.inf)
    for a, b in zip(path[:-1], path[1:]):
        seg = b - a
        ll = np.dot(seg, seg)
        if ll < 1e-14:
            d = np.linalg.norm(points - a, axis=1)
        else:
            t = np.clip(np.dot(points - a, seg) / ll, 0, 1)
            d = np.linalg.norm(points - (a + t[:, np.newaxis] * seg), axis=1)
        best = np.minimum(best, d)
    return best


def _nearest_radius(points, path, radii):
    """Radius at the nearest path vertex (the first of equal distances)."""
    out = np.empty(points.shape[0])
    for q in range(points.shape[0]):
        out[q] = radii[np.argmin(np.linalg.norm(path - points[q], axis=1))]
    return out


class HelicalTube(SDFPrimitive):  # sdf.py:1579-1721, paths.py:137-223
    def __init__(self, center, helix_radius, tube_radius_start, tube_radius_end, pitch, turns):
        c = np.array(center, dtype=np.float64)
        n = max(200, int(100 * float(turns)))
        theta = np.linspace(0, 2 * np.pi * float(turns), n)
        self.path = np.stack([c[0] + float(helix_radius) * np.cos(theta),
                              c[1] + float(helix_radius) * np.sin(theta),
                              c[2] + (theta / (2 * np.pi)) * float(pitch)], axis=1)
        t = np.linspace(0, 1, n)
        r0, r1 = float(tube_radius_start), float(tube_radius_end)
        self.radii = r0 + (r1 - r0) * t

    def sdf(self, points):
        points = np.asarray(points, dtype=np.float64)
        return _polyline_distance(points, self.path) - _nearest_radius(points, self.path,
                                                                       self.radii)


class SpiralHorn(SDFPrimitive):  # sdf.py:1392-1576, paths.py:30-134
    def __init__(self, center, throat_radius, mouth_radius, inner_spiral_radius,
                 outer_spiral_radius, turns, height, profile="exponential",
                 spiral_type="logarithmic"):
        c = np.array(center, dtype=np.float64)
        turns = float(turns)
        n = max(200, int(100 * turns))
        theta = np.linspace(0, 2 * np.pi * turns, n)
        ri, ro = float(inner_spiral_radius), float(outer_spiral_radius)
        if spiral_type == "logarithmic":
            r = ri * np.exp(np.log(ro / ri) / (2 * np.pi * turns) * theta)
        else:
            r = ri + (ro - ri) / (2 * np.pi * turns) * theta
        self.path = np.stack([c[0] + r * np.cos(theta), c[1] + r * np.sin(theta)], axis=1)
        t = np.linspace(0, 1, n)
        r0, r1 = float(throat_radius), float(mouth_radius)
        if profile == "exponential":
            self.radii = r0 * (r1 / r0) ** t
        elif profile == "linear":
            self.radii = r0 + (r1 - r0) * t
        else:
            self.radii = r0 / (1 - t * (1 - r0 / r1))
        self.height = float(height)

    def sdf(self, points):
        points = np.asarray(points, dtype=np.float64)
        xy, z = points[:, :2], points[:, 2]
        rd = _polyline_distance(xy, self.path) - _nearest_radius(xy, self.path, self.radii)
        zd = np.maximum(0, np.maximum(-z, z - self.height))
        inside = (z >= 0) & (z <= self.height)
        return np.where(inside, rd, np.sqrt(rd**2 + zd**2))


class _Smooth(SDFPrimitive):  # sdf.py:736-934
    sign = -1.0  # -1: smooth minimum (union); +1: smooth maximum

    def __init__(self, a, b, radius):
        self.a, self.b, self.radius = a, b, radius

    def _d2(self, points):
        return self.b.sdf(points)

    def sdf(self, points):
        d1, d2 = self.a.sdf(points), self._d2(points)
        h = np.clip(0.5 + 0.5 * (d2 - d1) / self.radius, 0, 1)
        mix = d2 * (1 - h) + d1 * h
        bump = self.radius * h * (1 - h)
        return mix + bump if self.sign > 0 else mix - bump


class SmoothUnion(_Smooth):
    sign = -1.0


class SmoothIntersection(_Smooth):
    sign = 1.0


class SmoothDifference(_Smooth):
    sign = 1.0

    def _d2(self, points):
        return -self.b.sdf(points)


class Union(SDFPrimitive):  # sdf.py:549-609
    def __init__(self, *children):
        self.children = children

    def sdf(self, points):
        if not self.children:
            return np.full(len(points), np.inf)
        return np.minimum.reduce([c.sdf(points) for c in self.children])


class Intersection(SDFPrimitive):  # sdf.py:612-682
    def __init__(self, *children):
        self.children = children

    def sdf(self, points):
        if not self.children:
            return np.full(len(points), -np.inf)
        return np.maximum.reduce([c.sdf(points) for c in self.children])


class Difference(SDFPrimitive):  # sdf.py:685-733
    def __init__(self, base, *subtracted):
        self.base = base
        self.subtracted = subtracted

    def sdf(self, points):
        r = self.base.sdf(points)
        for s in self.subtracted:
            r = np.maximum(r, -s.sdf(points))
        return r


class Translate(SDFPrimitive):  # sdf.py:1199-1236
    def __init__(self, child, offset):
        self.child = child
        self.offset = np.asarray(offset, dtype=np.float64)

    def sdf(self, points):
        return self.child.sdf(points - self.offset)


class Scale(SDFPrimitive):  # sdf.py:1239-1300
    def __init__(self, child, scale):
        self.child = child
        if np.isscalar(scale):
            self.scale = np.array([scale, scale, scale], dtype=np.float64)
            self.uniform = True
        else:
            self.scale = np.asarray(scale, dtype=np.float64)
            self.uniform = np.allclose(self.scale, self.scale[0])

    def sdf(self, points):
        d = self.child.sdf(points / self.scale)
        return d * self.scale[0] if self.uniform else d * np.min(self.scale)


def rotation_matrix(axis, angle):  # geometry/sdf.py:1151-1185
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


class Rotate(SDFPrimitive):  # geometry/sdf.py:1303-1355
    def __init__(self, child, axis=None, angle=None, matrix=None):
        self.child = child
        self.matrix = (np.asarray(matrix, dtype=np.float64) if matrix is not None
                       else rotation_matrix(np.asarray(axis), angle))
        self.inv_matrix = self.matrix.T

    def sdf(self, points):
        return self.child.sdf(np.asarray(points, dtype=np.float64) @ self.inv_matrix.T)


class HelmholtzResonator(SDFPrimitive):  # geometry/resonator.py:59-297
    def __init__(self, position, cavity_shape="box", cavity_size=(0.03, 0.03, 0.03),
                 neck_length=0.01, neck_radius=0.005, neck_direction=(0.0, 0.0, 1.0)):
        self.position = np.asarray(position, dtype=np.float64)
        nd = np.asarray(neck_direction, dtype=np.float64)
        self.neck_direction = nd / np.linalg.norm(nd)
        self.cavity_shape, self.cavity_size = cavity_shape, cavity_size
        if cavity_shape == "box":
            cav = Box(center=tuple(self.position), size=cavity_size)
            half = np.array(cavity_size, dtype=np.float64) / 2
            start = self.position + self.neck_direction * np.min(
                half / (np.abs(self.neck_direction) + 1e-10))
        elif cavity_shape == "sphere":
            cav = Sphere(center=tuple(self.position), radius=cavity_size[0])
            start = self.position + self.neck_direction * cavity_size[0]
        else:
            r, length = cavity_size
            ax = self.neck_direction * length
            cav = Cylinder(p1=tuple(self.position - ax / 2), p2=tuple(self.position + ax / 2),
                           radius=r)
            start = self.position + self.neck_direction * (length / 2)
        end = start + self.neck_direction * neck_length
        self._combined = Union(cav, Cylinder(p1=tuple(start), p2=tuple(end), radius=neck_radius))

    def sdf(self, points):
        return self._combined.sdf(points)


# ---------------------------------------------------------------------------
# Solver (core/solver.py:1441-2606, native step semantics)
class MaterializedGeometry:
    """geometry/material_assignment.py:48-198: an SDF whose inside is air,
    material regions in assignment order (ids 1, 2, ...), later ones
    overriding earlier ones, inside air only."""

    def __init__(self, geometry, default_material=None):
        self.geometry = geometry
        self.default_material = default_material
        self._regions = []

    def set_material(self, region, material):
        mid = len(self._regions) + 1
        if mid > 255:
            raise ValueError("Maximum of 255 material regions exceeded")
        self._regions.append((region, material, mid))
        return mid

    def voxelize_with_materials(self, grid):
        mask = self.geometry.voxelize(grid)
        ids = np.zeros(grid.shape, dtype=np.uint8)
        for region, _, mid in self._regions:
            ids[mask & region.voxelize(grid)] = mid
        return mask, ids

    def get_material_table(self):
        table = {0: self.default_material}
        for _, material, mid in self._regions:
            table[mid] = material
        return table


class Probe:
    def __init__(self, name, position):
        self.name, self.position, self.data = name, position, []


class FDTDSolver:
    def __init__(self, shape=None, resolution=None, grid=None, c=343.0, rho=1.2, courant=0.95,
                 backend="native", precision="f32"):
        self.grid = grid if grid is not None else UniformGrid(shape, resolution)
        self.shape = self.grid.shape
        self.dx = self.grid.min_spacing
        self.c, self.rho, self.precision = c, rho, precision
        dt_max = self.grid.min_spacing / (self.c * np.sqrt(3))
        self.dt = courant * dt_max
        self._nu = None
        if getattr(self.grid, "is_uniform", True):
            self._coeff_p = -self.rho * self.c**2 * self.dt / self.dx
            self._coeff_v = -self.dt / (self.rho * self.dx)
        else:  # base coefficients and float32 spacing arrays (solver.py:1587-1602)
            self._coeff_p = -self.rho * self.c**2 * self.dt
            self._coeff_v = -self.dt / self.rho
            self._nu = self.grid.get_spacing_arrays_for_stencil()
        self.real = np.float64 if precision == "f64" else np.float32
        self.p = np.zeros(self.shape, dtype=self.real)
        self.vx = np.zeros(self.shape, dtype=self.real)
        self.vy = np.zeros(self.shape, dtype=self.real)
        self.vz = np.zeros(self.shape, dtype=self.real)
        self.geometry = np.ones(self.shape, dtype=bool)
        self._geometry_set = False
        self._sources, self._probes, self._boundaries = [], {}, []
        self._materials = {}
        self._material_id = np.zeros(self.shape, dtype=np.uint8)
        self._ade = None
        self._step_count, self._time = 0, 0.0

    # -- setup (solver.py:1682-1990)
    def set_geometry(self, mask):
        if isinstance(mask, MaterializedGeometry):  # core/solver.py:1715-1760
            geo = mask
            mask, ids = geo.voxelize_with_materials(self.grid)
            for mid, material in geo.get_material_table().items():
                if mid == 0:
                    continue
                if mid not in self._materials:
                    self.register_material(material, material_id=mid)
                if np.any(ids == mid):
                    self.set_material_region(ids == mid, mid)
        elif isinstance(mask, SDFPrimitive):
            mask = mask.voxelize(self.grid)
        self.geometry = np.ascontiguousarray(mask, dtype=bool)
        self._geometry_set = True

    def _to_index(self, pos):
        if isinstance(pos, tuple) and len(pos) == 3 and any(
                isinstance(p, float) and p < max(self.shape) for p in pos):
            return tuple(int(round(p / self.dx)) for p in pos)
        return pos

    def add_source(self, source):
        if source.source_type == "point":
            source.position = self._to_index(source.position)
        self._sources.append(source)

    def add_probe(self, name, position):
        self._probes[name] = Probe(name, self._to_index(position))

    def add_boundary(self, b):
        b.initialize(self)
        self._boundaries.append(b)

    _PATTERNS = {"omni": 0.0, "subcardioid": 0.3, "cardioid": 0.5, "supercardioid": 0.63,
                 "hypercardioid": 0.75, "figure8": 1.0}  # core/solver.py:787-794
    _CORNERS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1),
                (1, 1, 1)]

    def add_microphone(self, position, name=None, pattern="omni", direction=None, up=None):
        """Microphone at a physical position (core/solver.py:853-963,
        1887-1965): grid position = position / dx; pattern coefficient or a
        custom gain(theta); unit direction."""
        if not hasattr(self, "_mics"):
            self._mics = {}
        d = np.array((1.0, 0.0, 0.0) if direction is None else direction, dtype=np.float64)
        d = d / np.linalg.norm(d)
        g = tuple(position[a] / self.dx for a in range(3))
        if not all(0 <= g[a] < self.shape[a] - 1 for a in range(3)):
            raise ValueError("microphone outside the domain")
        self._mics[name or f"mic_{len(self._mics)}"] = dict(
            g=g, direction=d, data=[],
            k=self._PATTERNS[pattern] if isinstance(pattern, str) else None,
            custom=None if isinstance(pattern, str) else pattern)

    def _trilinear_fp64(self, gx, gy, gz):
        """Microphone._compute_trilinear_weights (core/solver.py:965-1002)."""
        i0, j0, k0 = int(gx), int(gy), int(gz)
        fx, fy, fz = gx - i0, gy - j0, gz - k0
        w = [(1 - fx) * (1 - fy) * (1 - fz), fx * (1 - fy) * (1 - fz), (1 - fx) * fy * (1 - fz),
             fx * fy * (1 - fz), (1 - fx) * (1 - fy) * fz, fx * (1 - fy) * fz,
             (1 - fx) * fy * fz, fx * fy * fz]
        return [(i0 + a, j0 + b, k0 + c) for a, b, c in self._CORNERS], w

    def _record_mics(self):
        """FDTDSolver._record_microphones (core/solver.py:2441-2518): the
        native batch kernel when every microphone is omni, else
        Microphone.record for each (core/solver.py:1004-1179)."""
        mics = getattr(self, "_mics", {})
        directional = any(m["k"] != 0.0 for m in mics.values())
        one = np.float32(1.0)
        for m in mics.values():
            if not directional:  # microphones.cpp:16-118, float32 throughout
                gf = [np.float32(v) for v in m["g"]]
                i0 = [int(v) for v in gf]
                fx, fy, fz = (np.float32(v - np.float32(i)) for v, i in zip(gf, i0))
                w = [(one - fx) * (one - fy) * (one - fz), fx * (one - fy) * (one - fz),
                     (one - fx) * fy * (one - fz), fx * fy * (one - fz),
                     (one - fx) * (one - fy) * fz, fx * (one - fy) * fz, (one - fx) * fy * fz,
                     fx * fy * fz]
                s = np.float32(0.0)
                for q, (a, b, c) in enumerate(self._CORNERS):
                    s = np.float32(s + np.float32(w[q] * self.p[i0[0] + a, i0[1] + b, i0[2] + c]))
                m["data"].append(s)
                continue
            cells, w = self._trilinear_fp64(*m["g"])
            pressure = 0.0
            for cell, wq in zip(cells, w):
                pressure += wq * self.p[cell]
            if m["k"] == 0.0:
                m["data"].append(pressure)
                continue
            vel = []
            for axis, field in enumerate((self.vx, self.vy, self.vz)):
                g = list(m["g"])
                g[axis] -= 0.5
                n = field.shape
                g = [max(0.0, min(g[a], n[a] - 1.001)) for a in range(3)]
                vc, vw = self._trilinear_fp64(*g)
                v = 0.0
                for (i, j, k), wq in zip(vc, vw):
                    v += wq * field[min(i, n[0] - 1), min(j, n[1] - 1), min(k, n[2] - 1)]
                vel.append(v)
            d = m["direction"]
            Z = self.rho * self.c
            vd = vel[0] * d[0] + vel[1] * d[1] + vel[2] * d[2]
            if m["custom"] is not None:
                v_mag = np.sqrt(vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2)
                theta = np.arccos(np.clip(vd / v_mag, -1.0, 1.0)) if v_mag > 1e-20 else 0.0
                m["data"].append(pressure * m["custom"](theta))
            else:
                k = m["k"]
                m["data"].append((1 - k) * pressure + k * Z * vd)

    def get_mic_data(self):
        return {k: np.array(m["data"], dtype=np.float32) for k, m in getattr(self, "_mics", {}).items()}

    def register_material(self, material, material_id=None):
        if material_id is None:
            material_id = next(i for i in range(1, 256) if i not in self._materials)
        self._materials[material_id] = material
        self._ade = None
        return material_id

    def set_material_region(self, mask, material_id):
        self._material_id[mask] = material_id
        self._ade = None

    def set_material_box(self, material_id, x_range, y_range, z_range):
        m = np.zeros(self.shape, dtype=bool)
        m[x_range[0]:x_range[1], y_range[0]:y_range[1], z_range[0]:z_range[1]] = True
        self.set_material_region(m, material_id)

    # -- ADE tables (solver.py:2944-3083): one field per pole, Debye and
    # Lorentz numbered separately in registration order
    def _init_ade(self):
        R = self.real
        n = int(np.prod(self.shape))
        dt_r = R(self.dt)
        inv_dx = R(1.0 / self.dx)
        debye, lorentz = [], []
        for mid, mat in self._materials.items():
            rho_inf, k_inf = R(mat.rho_inf), R(mat.K_inf)
            for pole in mat.poles:
                tgt = 0 if pole.target == "density" else 1
                co = tuple(R(v) for v in pole.fdtd_coefficients(self.dt))
                # ade.cpp:263 / :420: coefficients formed in the kernel's precision
                cvel = R(R(-dt_r) / rho_inf) * inv_dx
                cpre = R(-k_inf) * dt_r
                e = dict(mid=mid, target=tgt, co=co, cvel=R(cvel), cpre=R(cpre))
                (debye if pole.is_debye else lorentz).append(e)
        for e in debye:
            e["J"] = np.zeros(n, dtype=R)
        for e in lorentz:
            e["J"] = np.zeros(n, dtype=R)
            e["Jp"] = np.zeros(n, dtype=R)
        self._ade = dict(debye=debye, lorentz=lorentz, inv_dx=inv_dx,
                         div=np.zeros(n, dtype=R))

    # -- stepping
    def _fns(self):
        L = lib()
        s = "f64" if self.precision == "f64" else "f32"
        return lambda name: getattr(L, f"orc_{name}_{s}")

    def _pml(self):
        dx = dy = dz = None
        for b in self._boundaries:
            dx, dy, dz = b.decay
        return dx, dy, dz

    def step(self):
        F = self._fns()
        nx, ny, nz = self.shape
        R = self.real
        cv, cp = R(self._coeff_v), R(self._coeff_p)
        p, vx, vy, vz = self.p, self.vx, self.vy, self.vz
        mat = self._material_id
        if self._materials and self._ade is None:
            self._init_ade()
        ade = self._ade if self._materials else None
        ncell = int(p.size)
        if ade:  # density poles, before the velocity update (solver.py:2138)
            for e in ade["debye"]:
                if e["target"] == 0:
                    F("ade_debye")(_ptr(e["J"]), _ptr(p), _ptr(mat), e["mid"], *e["co"], ncell)
            for e in ade["lorentz"]:
                if e["target"] == 0:
                    F("ade_lorentz")(_ptr(e["J"]), _ptr(e["Jp"]), _ptr(p), _ptr(mat), e["mid"],
                                     *e["co"], ncell)
        nu = None
        if self._nu is not None:
            nu = {k: np.ascontiguousarray(v, dtype=R) for k, v in self._nu.items()}
        if nu is not None:  # _step_native_nonuniform (solver.py:2104-2126)
            F("update_velocity_nu")(_ptr(p), _ptr(vx), _ptr(vy), _ptr(vz), nx, ny, nz, cv,
                                    _ptr(nu["inv_dx_face"]), _ptr(nu["inv_dy_face"]),
                                    _ptr(nu["inv_dz_face"]))
        else:
            F("update_velocity")(_ptr(p), _ptr(vx), _ptr(vy), _ptr(vz), nx, ny, nz, cv)
        if ade:
            for e in ade["debye"] + ade["lorentz"]:
                if e["target"] == 0:
                    F("ade_velocity_correction")(_ptr(vx), _ptr(vy), _ptr(vz), _ptr(e["J"]),
                                                 _ptr(mat), e["mid"], e["cvel"], nx, ny, nz)
        if self._geometry_set:
            F("apply_rigid")(_ptr(vx), _ptr(vy), _ptr(vz), _ptr(self.geometry.view(np.uint8)),
                             nx, ny, nz)
        if ade and any(e["target"] == 1 for e in ade["debye"] + ade["lorentz"]):
            if nu is not None:  # compute_divergence_nonuniform (solver.py:3161)
                F("divergence_nu")(_ptr(ade["div"]), _ptr(vx), _ptr(vy), _ptr(vz), nx, ny, nz,
                                   _ptr(nu["inv_dx_cell"]), _ptr(nu["inv_dy_cell"]),
                                   _ptr(nu["inv_dz_cell"]))
            else:
                F("divergence")(_ptr(ade["div"]), _ptr(vx), _ptr(vy), _ptr(vz), nx, ny, nz,
                                ade["inv_dx"])
            for e in ade["debye"]:
                if e["target"] == 1:
                    F("ade_debye")(_ptr(e["J"]), _ptr(ade["div"]), _ptr(mat), e["mid"], *e["co"],
                                   ncell)
            for e in ade["lorentz"]:
                if e["target"] == 1:
                    F("ade_lorentz")(_ptr(e["J"]), _ptr(e["Jp"]), _ptr(ade["div"]), _ptr(mat),
                                     e["mid"], *e["co"], ncell)
        if nu is not None:
            F("update_pressure_nu")(_ptr(p), _ptr(vx), _ptr(vy), _ptr(vz),
                                    _ptr(self.geometry.view(np.uint8)), nx, ny, nz, cp,
                                    _ptr(nu["inv_dx_cell"]), _ptr(nu["inv_dy_cell"]),
                                    _ptr(nu["inv_dz_cell"]))
        else:
            F("update_pressure")(_ptr(p), _ptr(vx), _ptr(vy), _ptr(vz),
                                 _ptr(self.geometry.view(np.uint8)), nx, ny, nz, cp)
        if ade:
            for e in ade["debye"] + ade["lorentz"]:
                if e["target"] == 1:
                    F("ade_pressure_correction")(_ptr(p), _ptr(e["J"]), _ptr(mat), e["mid"],
                                                 e["cpre"], ncell)
            p[~self.geometry] = 0.0
        for b in self._boundaries:  # boundary loops in order (solver.py:2040-2047)
            if isinstance(b, PML):
                F("pml_velocity")(_ptr(vx), _ptr(vy), _ptr(vz), *(_ptr(d) for d in b.decay),
                                  nx, ny, nz)
        for b in self._boundaries:
            if isinstance(b, PML):
                F("pml_pressure")(_ptr(p), *(_ptr(d) for d in b.decay), nx, ny, nz)
            else:
                b.apply_pressure(self)
        g = _ptr(self.geometry.view(np.uint8))
        for s in self._sources:
            if s.source_type == "membrane":  # solver.py:2389-2412
                val = s.waveform.waveform(np.array([self._time]), self.dt)[0]
                if s._w is None:
                    s._w = s.weights(self.grid)
                mask = (s._w > 0) & self.geometry
                if s.injection_type == "pressure":
                    f = p
                else:
                    f = {"x": vx, "y": vy, "z": vz}[s.normal_axis]
                f[mask] += val * s._w[mask]
                continue
            val = float(s.waveform(np.array([self._time]), self.dt)[0])
            kind, a, b_, c = self._src_desc(s)
            F("inject")(_ptr(p), g, nx, ny, nz, kind, a, b_, c, val)
        for pr in self._probes.values():
            pr.data.append(p[pr.position])
        self._record_mics()
        self._step_count += 1
        self._time += self.dt

    @staticmethod
    def _src_desc(s):
        if s.source_type == "point":
            return (0, *s.position)
        return (1, s.position["axis"], s.position["index"], 0)

    def run_steps(self, n):
        """n steps of the plain path through one C call (no ADE, one PML);
        with ADE materials or microphones, step by step."""
        if (self._materials or getattr(self, "_mics", None) or self._nu is not None
                or any(not isinstance(b, PML) for b in self._boundaries)
                or any(s.source_type == "membrane" for s in self._sources)):
            for _ in range(n):
                self.step()
            return
        assert len(self._boundaries) <= 1
        nx, ny, nz = self.shape
        R = self.real
        vals = np.zeros((n, max(1, len(self._sources))), dtype=np.float64)
        t = self._time
        for q in range(n):
            for si, s in enumerate(self._sources):
                vals[q, si] = s.waveform(np.array([t]), self.dt)[0]
            t += self.dt
        src = np.array([self._src_desc(s) for s in self._sources] or [[0, 0, 0, 0]],
                       dtype=np.int32)
        probes = list(self._probes.values())
        cells = np.array([np.ravel_multi_index(pr.position, self.shape) for pr in probes] or [0],
                         dtype=np.int64)
        trace = np.zeros((n, max(1, len(probes))), dtype=R)
        dx, dy, dz = self._pml()
        Plan = _PlanD if self.precision == "f64" else _PlanF
        plan = Plan(nx, ny, nz, R(self._coeff_v), R(self._coeff_p),
                    _ptr(self.geometry.view(np.uint8)) if self._geometry_set else None,
                    _ptr(dx), _ptr(dy), _ptr(dz), len(self._sources), _ptr(src),
                    len(probes), _ptr(cells))
        self._fns()("run_plain")(ctypes.addressof(plan), _ptr(self.p), _ptr(self.vx),
                                 _ptr(self.vy), _ptr(self.vz), n, _ptr(vals), _ptr(trace))
        for qi, pr in enumerate(probes):
            pr.data.extend(trace[:, qi].tolist())
        self._step_count += n
        for _ in range(n):
            self._time += self.dt

    def get_probe_data(self, name=None):
        names = [name] if name is not None else list(self._probes)
        return {k: np.array(self._probes[k].data, dtype=np.float32) for k in names}


def boundary_faces(geometry, axis):
    """precompute_boundary_cells lists (boundaries.cpp:13-64) for one axis."""
    g = np.ascontiguousarray(geometry, dtype=np.uint8)
    nx, ny, nz = g.shape
    f = lib().orc_boundary_faces_f32
    n = f(g.ctypes.data, nx, ny, nz, axis, None)
    out = np.zeros(n, dtype=np.int32)
    f(g.ctypes.data, nx, ny, nz, axis, out.ctypes.data)
    return out


api = None


def make_api():
    """Namespace with the reference API names, for tests/golden/cases.py."""
    import types
    return types.SimpleNamespace(
        FDTDSolver=FDTDSolver, UniformGrid=UniformGrid, NonuniformGrid=NonuniformGrid, PML=PML,
        ABCFirstOrder=ABCFirstOrder, RadiationImpedance=RadiationImpedance,
        CircularMembraneSource=CircularMembraneSource,
        RectangularMembraneSource=RectangularMembraneSource,
        GaussianPulse=GaussianPulse,
        Box=Box, Sphere=Sphere, Cylinder=Cylinder, Union=Union, Intersection=Intersection,
        Difference=Difference, HelmholtzResonator=HelmholtzResonator, Pole=Pole,
        Cone=Cone, Horn=Horn, HelicalTube=HelicalTube, SpiralHorn=SpiralHorn,
        SmoothUnion=SmoothUnion, SmoothIntersection=SmoothIntersection,
        SmoothDifference=SmoothDifference,
        PoleType=PoleType, SimpleMaterial=SimpleMaterial,
        MaterializedGeometry=MaterializedGeometry)
