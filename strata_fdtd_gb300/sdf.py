"""SDF primitives and CSG, evaluated on the GPU (geometry/sdf.py of
rjwalters/strata-fdtd).

Each shape compiles to a short stack program (``sf_sdf_node``, see
include/sf_gb300.h) that the voxelisation kernel runs per cell in FP64 with
the reference's operation order, so ``voxelize`` returns the same mask as the
reference's NumPy ``SDFPrimitive.voxelize`` (sdf.py:99-125).  Shape
construction (centres, sizes, unit axes, lengths) runs on the host in the
reference's own NumPy arithmetic, so the constants the kernel sees are the
reference's constants.

Supported: Box, Sphere, Cylinder, Cone, Horn (conical, exponential,
hyperbolic, tractrix), SpiralHorn, HelicalTube, Union, Intersection,
Difference, SmoothUnion, SmoothIntersection, SmoothDifference, Translate,
Scale, Rotate (axis-angle or matrix, rotate_x/y/z), HelmholtzResonator
(geometry/resonator.py).
"""
from __future__ import annotations

import ctypes
from functools import cached_property

import numpy as np

from . import _native

OP_BOX, OP_SPHERE, OP_CYLINDER, OP_CONE, OP_HORN, OP_TUBE, OP_SPIRAL = 1, 2, 3, 4, 5, 6, 7
OP_UNION, OP_INTERSECTION, OP_DIFFERENCE = 10, 11, 12
OP_SMOOTH_UNION, OP_SMOOTH_INTERSECTION, OP_SMOOTH_DIFFERENCE = 13, 14, 15
OP_PUSH_TRANSLATE, OP_PUSH_SCALE, OP_POP_POINT, OP_SCALE_DIST, OP_NEGATE = 20, 21, 22, 23, 24
OP_PUSH_ROTATE, OP_ROTATE_ROW2, OP_DATA = 25, 26, 27


def _node(op, n=0, a=(0.0, 0.0, 0.0), b=(0.0, 0.0, 0.0), s0=0.0, s1=0.0):
    nd = _native.SfSdfNode()
    nd.op, nd.n = op, n
    for q in range(3):
        nd.a[q] = float(a[q])
        nd.b[q] = float(b[q])
    nd.s0, nd.s1 = float(s0), float(s1)
    return nd


class SDFPrimitive:
    """Base class: negative distance inside, positive outside."""

    def _emit(self, prog: list) -> None:
        raise NotImplementedError(f"{type(self).__name__} is not supported by the GPU voxeliser")

    def program(self):
        prog: list = []
        self._emit(prog)
        arr = (_native.SfSdfNode * len(prog))(*prog)
        return arr, len(prog)

    # -- evaluation ---------------------------------------------------------
    def voxelize_device(self, grid, invert: bool = False, out=None, stream=None):
        """Voxelise on the GPU into a torch.uint8 CUDA tensor of grid.shape
        (1 = inside, or 1 = outside when ``invert``)."""
        import torch

        nx, ny, nz = grid.shape
        if out is None:
            out = torch.empty((nx, ny, nz), dtype=torch.uint8, device="cuda")
        prog, n = self.program()
        st = (stream or torch.cuda.current_stream()).cuda_stream
        if getattr(grid, "is_uniform", True):
            _native.check(_native.load().sf_voxelize(ctypes.addressof(prog), n, nx, ny, nz,
                                                     float(grid.min_spacing), int(invert),
                                                     out.data_ptr(), st), "sf_voxelize")
        else:  # the nonuniform grid's own cell centres
            cs = [np.ascontiguousarray(c, dtype=np.float64)
                  for c in (grid.x_coords, grid.y_coords, grid.z_coords)]
            ptrs = (ctypes.c_void_p * 3)(*[c.ctypes.data for c in cs])
            _native.check(_native.load().sf_voxelize_coords(ctypes.addressof(prog), n, nx, ny,
                                                            nz, ptrs, int(invert),
                                                            out.data_ptr(), st),
                          "sf_voxelize_coords")
        return out

    def voxelize(self, grid) -> np.ndarray:
        """Boolean mask of grid.shape, True inside (geometry/sdf.py:99-125)."""
        return self.voxelize_device(grid).cpu().numpy().astype(bool)

    def sdf(self, points) -> np.ndarray:
        """Signed distance at an (N, 3) array of points, evaluated on the GPU."""
        import torch

        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError(f"points must be Nx3 array, got shape {pts.shape}")
        dev = torch.from_numpy(pts).cuda()
        out = torch.empty(len(pts), dtype=torch.float64, device="cuda")
        prog, n = self.program()
        lib = _native.load()
        _native.check(lib.sf_sdf_eval(ctypes.addressof(prog), n, dev.data_ptr(), len(pts),
                                      out.data_ptr(), torch.cuda.current_stream().cuda_stream),
                      "sf_sdf_eval")
        return out.cpu().numpy()

    def contains(self, points) -> np.ndarray:
        return self.sdf(points) <= 0

    # -- fluent transforms (sdf.py:127-229) ----------------------------------
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


class Box(SDFPrimitive):
    """Axis-aligned box from (center, size) or (min_corner, max_corner)."""

    def __init__(self, center=None, size=None, min_corner=None, max_corner=None):
        if center is not None and size is not None:
            self.center = np.array(center, dtype=np.float64)
            self.size = np.array(size, dtype=np.float64)
        elif min_corner is not None and max_corner is not None:
            lo = np.array(min_corner, dtype=np.float64)
            hi = np.array(max_corner, dtype=np.float64)
            self.center = (lo + hi) / 2
            self.size = hi - lo
        else:
            raise ValueError("Must provide either (center, size) or (min_corner, max_corner)")
        if np.any(self.size <= 0):
            raise ValueError(f"Box size must be positive, got {self.size}")

    def _emit(self, prog):
        prog.append(_node(OP_BOX, a=self.center, b=self.size))

    @property
    def bounding_box(self):
        h = self.size / 2
        return self.center - h, self.center + h


class Sphere(SDFPrimitive):
    def __init__(self, center, radius):
        self.center = np.array(center, dtype=np.float64)
        self.radius = float(radius)
        if self.radius <= 0:
            raise ValueError(f"Sphere radius must be positive, got {self.radius}")

    def _emit(self, prog):
        prog.append(_node(OP_SPHERE, a=self.center, s0=self.radius))

    @property
    def bounding_box(self):
        r = np.array([self.radius] * 3)
        return self.center - r, self.center + r


class Cylinder(SDFPrimitive):
    """Capped cylinder between p1 and p2 (sdf.py:341-433)."""

    def __init__(self, p1, p2, radius):
        self.p1 = np.array(p1, dtype=np.float64)
        self.p2 = np.array(p2, dtype=np.float64)
        self.radius = float(radius)
        if self.radius <= 0:
            raise ValueError(f"Cylinder radius must be positive, got {self.radius}")
        self.axis = self.p2 - self.p1
        self.length = np.linalg.norm(self.axis)
        if self.length == 0:
            raise ValueError("Cylinder endpoints must be distinct")
        self.axis_normalized = self.axis / self.length

    def _emit(self, prog):
        prog.append(_node(OP_CYLINDER, a=self.p1, b=self.axis_normalized, s0=self.length,
                          s1=self.radius))

    @property
    def bounding_box(self):
        r = np.array([self.radius] * 3)
        return np.minimum(self.p1, self.p2) - r, np.maximum(self.p1, self.p2) + r


class Cone(SDFPrimitive):
    """Frustum from radius r1 at p1 to r2 at p2, either radius may be zero
    (sdf.py:436-541)."""

    def __init__(self, p1, p2, r1, r2):
        self.p1 = np.array(p1, dtype=np.float64)
        self.p2 = np.array(p2, dtype=np.float64)
        self.r1, self.r2 = float(r1), float(r2)
        if self.r1 < 0 or self.r2 < 0:
            raise ValueError(f"Cone radii must be non-negative, got r1={r1}, r2={r2}")
        if self.r1 == 0 and self.r2 == 0:
            raise ValueError("Cone cannot have both radii zero")
        self.axis = self.p2 - self.p1
        self.length = np.linalg.norm(self.axis)
        if self.length == 0:
            raise ValueError("Cone endpoints must be distinct")
        self.axis_normalized = self.axis / self.length

    def _emit(self, prog):
        prog.append(_node(OP_CONE, a=self.p1, b=self.axis_normalized, s0=self.length,
                          s1=self.r1))
        prog.append(_node(OP_DATA, a=(self.r2 - self.r1, 0.0, 0.0)))

    @property
    def bounding_box(self):
        r = np.array([max(self.r1, self.r2)] * 3)
        return np.minimum(self.p1, self.p2) - r, np.maximum(self.p1, self.p2) + r


_HORN_PROFILES = ("conical", "exponential", "hyperbolic", "tractrix")


class Horn(SDFPrimitive):
    """Horn from throat to mouth, a surface of revolution whose radius
    follows a conical, exponential, hyperbolic or tractrix flare
    (sdf.py:937-1148)."""

    def __init__(self, throat_position, mouth_position, throat_radius, mouth_radius,
                 profile="exponential"):
        if profile not in _HORN_PROFILES:
            raise ValueError(f"profile must be one of {set(_HORN_PROFILES)}, got '{profile}'")
        self.throat_position = np.array(throat_position, dtype=np.float64)
        self.mouth_position = np.array(mouth_position, dtype=np.float64)
        self.throat_radius, self.mouth_radius = float(throat_radius), float(mouth_radius)
        self.profile = profile
        if self.throat_radius <= 0 or self.mouth_radius <= 0:
            raise ValueError(f"Horn radii must be positive, got throat={throat_radius}, "
                             f"mouth={mouth_radius}")
        axis = self.mouth_position - self.throat_position
        self._length = np.linalg.norm(axis)
        if self._length == 0:
            raise ValueError("Horn throat and mouth positions must be distinct")
        self._axis = axis / self._length
        # flare constant from the area ratio (sdf.py:1013-1037)
        a0 = np.pi * self.throat_radius ** 2
        am = np.pi * self.mouth_radius ** 2
        L = self._length
        if profile == "conical":  # A = A0 (1 + m t)^2
            self._m = np.sqrt(am / a0) - 1
        elif profile == "exponential":  # A = A0 exp(2 alpha x)
            self._alpha = np.log(am / a0) / (2 * L)
        elif profile == "hyperbolic":  # A = A0 cosh^2(alpha x)
            self._alpha = np.arccosh(np.sqrt(am / a0)) / L
        else:  # A = A0 / cos^4(x / R)
            self._R = L / np.arccos(np.power(a0 / am, 0.25))

    def _flare(self):
        return {"conical": getattr(self, "_m", 0.0), "exponential": getattr(self, "_alpha", 0.0),
                "hyperbolic": getattr(self, "_alpha", 0.0),
                "tractrix": getattr(self, "_R", 0.0)}[self.profile]

    def radius_at_position(self, t):
        """Radius at normalised axial position t (0 throat, 1 mouth)."""
        t = np.asarray(t)
        x = t * self._length
        if self.profile == "conical":
            return self.throat_radius * (1 + self._m * t)
        if self.profile == "exponential":
            return self.throat_radius * np.exp(self._alpha * x)
        if self.profile == "hyperbolic":
            return self.throat_radius * np.cosh(self._alpha * x)
        return self.throat_radius / np.cos(x / self._R) ** 2

    @property
    def cutoff_frequency(self) -> float:
        """Low-frequency cutoff in Hz at c = 343 m/s (sdf.py:1061-1083)."""
        c = 343.0
        if self.profile == "conical":
            return c / (2 * np.pi * self._length)
        if self.profile in ("exponential", "hyperbolic"):
            return c * self._alpha / (2 * np.pi)
        return c / (4 * self._R)

    def _emit(self, prog):
        prog.append(_node(OP_HORN, n=_HORN_PROFILES.index(self.profile), a=self.throat_position,
                          b=self._axis, s0=self._length, s1=self.throat_radius))
        prog.append(_node(OP_DATA, a=(float(self._flare()), 0.0, 0.0)))

    @property
    def bounding_box(self):
        r = np.array([self.mouth_radius] * 3)
        return (np.minimum(self.throat_position, self.mouth_position) - r,
                np.maximum(self.throat_position, self.mouth_position) + r)


def conical_horn(throat_pos, mouth_pos, throat_r, mouth_r) -> Horn:
    return Horn(throat_pos, mouth_pos, throat_r, mouth_r, "conical")


def exponential_horn(throat_pos, mouth_pos, throat_r, mouth_r) -> Horn:
    return Horn(throat_pos, mouth_pos, throat_r, mouth_r, "exponential")


def hyperbolic_horn(throat_pos, mouth_pos, throat_r, mouth_r) -> Horn:
    return Horn(throat_pos, mouth_pos, throat_r, mouth_r, "hyperbolic")


def tractrix_horn(throat_pos, mouth_pos, throat_r, mouth_r) -> Horn:
    return Horn(throat_pos, mouth_pos, throat_r, mouth_r, "tractrix")


def _emit_path(prog, op, vertices, radii, s0=0.0):
    """A path shape: the header, then one node per vertex with the vertex, its
    radius and its segment to the next vertex with the squared length (in the
    reference's NumPy arithmetic, paths.py:276-281)."""
    v = np.asarray(vertices, dtype=np.float64)
    prog.append(_node(op, n=len(v), s0=s0))
    for q in range(len(v)):
        a = tuple(v[q]) + (0.0,) * (3 - v.shape[1])
        if q + 1 < len(v):
            seg = v[q + 1] - v[q]
            ll = np.dot(seg, seg)
            b = tuple(seg) + (0.0,) * (3 - v.shape[1])
        else:
            b, ll = (0.0, 0.0, 0.0), 0.0
        prog.append(_node(OP_DATA, a=a, b=b, s0=float(radii[q]), s1=float(ll)))


class SpiralHorn(SDFPrimitive):
    """Horn along a spiral in the xy plane, extruded over 0 <= z <= height:
    distance to the sampled spiral minus the radius at the nearest sample
    (sdf.py:1392-1576)."""

    def __init__(self, center, throat_radius, mouth_radius, inner_spiral_radius,
                 outer_spiral_radius, turns, height, profile="exponential",
                 spiral_type="logarithmic"):
        from .paths import SpiralPath

        self.center_2d = np.array(center, dtype=np.float64)
        self.throat_radius, self.mouth_radius = float(throat_radius), float(mouth_radius)
        self.inner_spiral_radius = float(inner_spiral_radius)
        self.outer_spiral_radius = float(outer_spiral_radius)
        self.turns, self.height = float(turns), float(height)
        self.profile, self.spiral_type = profile, spiral_type
        if self.throat_radius <= 0 or self.mouth_radius <= 0:
            raise ValueError("Throat and mouth radii must be positive")
        if self.height <= 0:
            raise ValueError("Height must be positive")
        if profile not in ("exponential", "linear", "hyperbolic"):
            raise ValueError("profile must be 'exponential', 'linear', or 'hyperbolic'")
        self.spiral = SpiralPath(center=self.center_2d, inner_radius=self.inner_spiral_radius,
                                 outer_radius=self.outer_spiral_radius, turns=self.turns,
                                 spiral_type=spiral_type)
        n = max(200, int(100 * self.turns))  # about 100 samples per turn
        self.path_2d = self.spiral.sample_points(n)
        t = np.linspace(0, 1, n)
        r0, r1 = self.throat_radius, self.mouth_radius
        if profile == "exponential":
            self.radii = r0 * (r1 / r0) ** t
        elif profile == "linear":
            self.radii = r0 + (r1 - r0) * t
        else:
            self.radii = r0 / (1 - t * (1 - r0 / r1))

    def _emit(self, prog):
        _emit_path(prog, OP_SPIRAL, self.path_2d, self.radii, s0=self.height)

    @property
    def bounding_box(self):
        e = self.outer_spiral_radius + max(self.throat_radius, self.mouth_radius)
        return (np.array([self.center_2d[0] - e, self.center_2d[1] - e, 0.0]),
                np.array([self.center_2d[0] + e, self.center_2d[1] + e, self.height]))


class HelicalTube(SDFPrimitive):
    """Tube along a helix, its radius tapering linearly from start to end:
    distance to the sampled helix minus the radius at the nearest sample
    (sdf.py:1579-1721)."""

    def __init__(self, center, helix_radius, tube_radius_start, tube_radius_end, pitch, turns):
        from .paths import HelixPath

        self.center = np.array(center, dtype=np.float64)
        self.helix_radius = float(helix_radius)
        self.tube_radius_start, self.tube_radius_end = float(tube_radius_start), float(tube_radius_end)
        self.pitch, self.turns = float(pitch), float(turns)
        if self.helix_radius <= 0:
            raise ValueError("helix_radius must be positive")
        if self.tube_radius_start <= 0 or self.tube_radius_end <= 0:
            raise ValueError("tube radii must be positive")
        if self.pitch <= 0:
            raise ValueError("pitch must be positive")
        if self.turns <= 0:
            raise ValueError("turns must be positive")
        self.helix = HelixPath(center=self.center, radius=self.helix_radius, pitch=self.pitch,
                               turns=self.turns)
        n = max(200, int(100 * self.turns))
        self.path_3d = self.helix.sample_points(n)
        t = np.linspace(0, 1, n)
        self.tube_radii = (self.tube_radius_start
                           + (self.tube_radius_end - self.tube_radius_start) * t)

    def _emit(self, prog):
        _emit_path(prog, OP_TUBE, self.path_3d, self.tube_radii)

    @property
    def bounding_box(self):
        e = self.helix_radius + max(self.tube_radius_start, self.tube_radius_end)
        return (np.array([self.center[0] - e, self.center[1] - e, self.center[2]]),
                np.array([self.center[0] + e, self.center[1] + e,
                          self.center[2] + self.helix.total_height]))


def _emit_fold(prog, children, op):
    """Emit an n-ary CSG node as a left fold of two-operand steps
    (c0, c1, op, c2, op, ...): the reference folds its children in the same
    order, and the evaluation stack then grows with the tree's depth only,
    not with the number of children."""
    if not children:
        prog.append(_node(op, n=0))
        return
    children[0]._emit(prog)
    if len(children) == 1:
        prog.append(_node(op, n=1))
    for c in children[1:]:
        c._emit(prog)
        prog.append(_node(op, n=2))


class CSGNode(SDFPrimitive):
    pass


class Union(CSGNode):
    """min over children (sdf.py:549-609)."""

    def __init__(self, *children):
        self.children = children

    def _emit(self, prog):
        _emit_fold(prog, self.children, OP_UNION)

    @cached_property
    def bounding_box(self):
        if not self.children:
            return np.array([np.inf] * 3), np.array([-np.inf] * 3)
        return (np.minimum.reduce([c.bounding_box[0] for c in self.children]),
                np.maximum.reduce([c.bounding_box[1] for c in self.children]))


class Intersection(CSGNode):
    """max over children (sdf.py:612-682)."""

    def __init__(self, *children):
        self.children = children

    def _emit(self, prog):
        _emit_fold(prog, self.children, OP_INTERSECTION)

    @cached_property
    def bounding_box(self):
        if not self.children:
            return np.array([-np.inf] * 3), np.array([np.inf] * 3)
        lo = np.maximum.reduce([c.bounding_box[0] for c in self.children])
        hi = np.minimum.reduce([c.bounding_box[1] for c in self.children])
        if np.any(lo > hi):
            return np.array([np.inf] * 3), np.array([-np.inf] * 3)
        return lo, hi


class Difference(CSGNode):
    """max(base, -s1, -s2, ...) (sdf.py:685-733)."""

    def __init__(self, base, *subtracted):
        self.base = base
        self.subtracted = subtracted

    def _emit(self, prog):
        _emit_fold(prog, (self.base,) + tuple(self.subtracted), OP_DIFFERENCE)

    @cached_property
    def bounding_box(self):
        return self.base.bounding_box


class SmoothUnion(CSGNode):
    """Union of two shapes blended over ``radius`` by the polynomial smooth
    minimum (sdf.py:736-800)."""

    def __init__(self, a, b, radius):
        if radius <= 0:
            raise ValueError(f"radius must be positive, got {radius}")
        self.a, self.b, self.radius = a, b, radius

    def _emit(self, prog):
        self.a._emit(prog)
        self.b._emit(prog)
        prog.append(_node(OP_SMOOTH_UNION, s0=self.radius))

    @cached_property
    def bounding_box(self):
        (la, ha), (lb, hb) = self.a.bounding_box, self.b.bounding_box
        r = np.array([self.radius] * 3)
        return np.minimum(la, lb) - r, np.maximum(ha, hb) + r


class SmoothIntersection(CSGNode):
    """Intersection blended by the polynomial smooth maximum
    (sdf.py:803-877)."""

    def __init__(self, a, b, radius):
        if radius <= 0:
            raise ValueError(f"radius must be positive, got {radius}")
        self.a, self.b, self.radius = a, b, radius

    def _emit(self, prog):
        self.a._emit(prog)
        self.b._emit(prog)
        prog.append(_node(OP_SMOOTH_INTERSECTION, s0=self.radius))

    @cached_property
    def bounding_box(self):
        (la, ha), (lb, hb) = self.a.bounding_box, self.b.bounding_box
        r = np.array([self.radius] * 3)
        lo, hi = np.maximum(la, lb) + r, np.minimum(ha, hb) - r
        if np.any(lo > hi):
            return np.array([np.inf] * 3), np.array([-np.inf] * 3)
        return lo, hi


class SmoothDifference(CSGNode):
    """``base`` minus ``subtracted``, blended as the smooth intersection with
    the subtracted shape's complement (sdf.py:880-934)."""

    def __init__(self, base, subtracted, radius):
        if radius <= 0:
            raise ValueError(f"radius must be positive, got {radius}")
        self.base, self.subtracted, self.radius = base, subtracted, radius

    def _emit(self, prog):
        self.base._emit(prog)
        self.subtracted._emit(prog)
        prog.append(_node(OP_SMOOTH_DIFFERENCE, s0=self.radius))

    @cached_property
    def bounding_box(self):
        lo, hi = self.base.bounding_box
        r = np.array([self.radius] * 3)
        return lo - r, hi + r


class Transform(SDFPrimitive):
    def __init__(self, child):
        self.child = child


class Translate(Transform):
    """Evaluate the child at point - offset (sdf.py:1199-1236)."""

    def __init__(self, child, offset):
        super().__init__(child)
        self.offset = np.asarray(offset, dtype=np.float64)
        if self.offset.shape != (3,):
            raise ValueError(f"offset must be a 3-element vector, got shape {self.offset.shape}")

    def _emit(self, prog):
        prog.append(_node(OP_PUSH_TRANSLATE, a=self.offset))
        self.child._emit(prog)
        prog.append(_node(OP_POP_POINT))

    @property
    def bounding_box(self):
        lo, hi = self.child.bounding_box
        return lo + self.offset, hi + self.offset


class Scale(Transform):
    """Evaluate the child at point / scale, scale the distance by scale[0]
    (uniform) or min(scale) (sdf.py:1239-1300)."""

    def __init__(self, child, scale):
        super().__init__(child)
        if np.isscalar(scale):
            self.scale = np.array([scale, scale, scale], dtype=np.float64)
            self.uniform = True
        else:
            self.scale = np.asarray(scale, dtype=np.float64)
            self.uniform = np.allclose(self.scale, self.scale[0])
        if self.scale.shape != (3,):
            raise ValueError("scale must be scalar or 3-element vector")
        if np.any(self.scale <= 0):
            raise ValueError(f"scale factors must be positive, got {self.scale}")

    def _emit(self, prog):
        prog.append(_node(OP_PUSH_SCALE, a=self.scale))
        self.child._emit(prog)
        prog.append(_node(OP_POP_POINT))
        f = self.scale[0] if self.uniform else np.min(self.scale)
        prog.append(_node(OP_SCALE_DIST, s0=float(f)))

    @property
    def bounding_box(self):
        lo, hi = self.child.bounding_box
        return lo * self.scale, hi * self.scale


def rotation_matrix(axis, angle):
    """Rodrigues' rotation matrix I + sin(a) K + (1 - cos(a)) K K for the
    normalised axis (geometry/sdf.py:1151-1185): the reference's NumPy
    expression, so the matrix entries are the reference's."""
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


class Rotate(Transform):
    """Evaluate the child at the inversely rotated point, point @ R
    (geometry/sdf.py:1303-1390): each coordinate the sum
    ((p0 m0 + p1 m1) + p2 m2) of a row of R^T.  NumPy's matrix product
    goes through BLAS, whose summation order is its own: for a rotation that
    is not a multiple of 90 degrees about a coordinate axis, cells within
    rounding (about 1e-16 m) of a surface may fall on the other side."""

    def __init__(self, child, axis=None, angle=None, matrix=None):
        super().__init__(child)
        if matrix is not None:
            self.matrix = np.asarray(matrix, dtype=np.float64)
            if self.matrix.shape != (3, 3):
                raise ValueError(f"matrix must be 3x3, got shape {self.matrix.shape}")
        elif axis is not None and angle is not None:
            self.matrix = rotation_matrix(np.asarray(axis), angle)
        else:
            raise ValueError("Must provide either (axis, angle) or matrix")
        self.inv_matrix = self.matrix.T

    def _emit(self, prog):
        m = self.inv_matrix  # point' = point @ inv.T: coordinate i = sum_j p_j inv[i, j]
        prog.append(_node(OP_PUSH_ROTATE, a=m[0], b=m[1]))
        prog.append(_node(OP_ROTATE_ROW2, a=m[2]))
        self.child._emit(prog)
        prog.append(_node(OP_POP_POINT))

    @property
    def bounding_box(self):
        lo, hi = self.child.bounding_box
        corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1])
                            for z in (lo[2], hi[2])])
        rc = corners @ self.matrix.T
        return rc.min(axis=0), rc.max(axis=0)
