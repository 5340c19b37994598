"""FDTDSolver on the GB300: the reference API (core/solver.py of
rjwalters/strata-fdtd) over the sf_* C ABI.

What stays as in the reference: constructor arguments, dt and the update
coefficients (core/solver.py:1576-1602, same FP64 expressions), the public
NumPy fields ``p``, ``vx``, ``vy``, ``vz`` and ``geometry``, source and probe
handling (index vs metre positions, :1782-1885), the FP64 ``_time``
accumulation (:2071-2072), ``step``/``run`` semantics (:2003-2077,
:2520-2606) and ``get_probe_data`` returning float32 arrays.

What changes: the fields live in HBM as two ping-pong sets of CUDA tensors;
one fused kernel per time step does the velocity, rigid-wall, pressure, PML,
ADE, source and probe work; ``run`` issues all steps of a call in one C-ABI
call with the waveform values precomputed (the reference's NumPy
expression at the same FP64 times, elementwise-identical) and the probe
traces kept on the device until read.

Host/device coherence: reading ``solver.p`` (etc.) copies the current device
state into one persistent NumPy array per field, and marks it as possibly
modified, so the next step uploads it again -- in-place edits such as
``solver.p[i, j, k] = 1.0`` behave as they do on the reference.

There is no CPU fallback: without a CUDA device or the compiled library the
constructor raises.
"""
from __future__ import annotations

import ctypes
import warnings
from dataclasses import dataclass, field
from typing import Literal

import numpy as np

from . import _native
from .boundaries import PML, ABCFirstOrder, RadiationImpedance, RigidBoundary
from .grid import UniformGrid
from .sdf import SDFPrimitive

_FIELDS = ("p", "vx", "vy", "vz")
_MAX_CHUNK = 1 << 16  # steps per C-ABI call inside run()


@dataclass
class GaussianPulse:
    """Gaussian-modulated sinusoid (core/solver.py:152-207)."""

    position: tuple | dict
    frequency: float
    bandwidth: float | None = None
    amplitude: float = 1.0
    source_type: Literal["point", "plane"] = "point"

    def __post_init__(self):
        if self.bandwidth is None:
            self.bandwidth = 2.0 * self.frequency

    def waveform(self, t, dt):
        sigma = 1.0 / (np.pi * self.bandwidth)
        t0 = 4.0 * sigma
        envelope = np.exp(-((t - t0) ** 2) / (2 * sigma**2))
        carrier = np.sin(2 * np.pi * self.frequency * (t - t0))
        return self.amplitude * envelope * carrier


@dataclass
class Probe:
    """Pressure probe at a grid cell (core/solver.py:758-781).  Samples are
    held on the device and copied out when ``data`` or ``get_data`` is read."""

    name: str
    position: tuple
    _samples: list = field(default_factory=list, repr=False)
    _solver: object = field(default=None, repr=False)

    @property
    def data(self) -> list:
        if self._solver is not None:
            self._solver._flush_traces()
        return self._samples

    def record(self, pressure: float) -> None:
        self._samples.append(float(pressure))

    def get_data(self) -> np.ndarray:
        return np.array(self.data, dtype=np.float32)

    def clear(self) -> None:
        if self._solver is not None:
            self._solver._flush_traces()
        self._samples.clear()


def step_coefficients(grid, c: float, rho: float, courant: float):
    """dt, coeff_v, coeff_p with the FP64 expressions of core/solver.py:1576-1591;
    on a nonuniform grid the base coefficients without the 1/dx factor."""
    dx = grid.min_spacing
    dt_max = grid.min_spacing / (c * np.sqrt(3))
    dt = courant * dt_max
    if not getattr(grid, "is_uniform", True):
        return dt, -dt / rho, -rho * c**2 * dt
    coeff_p = -rho * c**2 * dt / dx
    coeff_v = -dt / (rho * dx)
    return dt, coeff_v, coeff_p


def _fresh_host_array(shape) -> np.ndarray:
    """A new float32 array for a snapshot: anonymous memory asking for
    transparent huge pages when it is large (fewer page faults when it is
    first written), else np.empty."""
    n = int(np.prod(shape))
    if n * 4 < (64 << 20):
        return np.empty(shape, dtype=np.float32)
    import mmap
    mm = mmap.mmap(-1, n * 4)
    if hasattr(mmap, "MADV_HUGEPAGE"):
        try:
            mm.madvise(mmap.MADV_HUGEPAGE)
        except OSError:
            pass
    return np.frombuffer(mm, dtype=np.float32, count=n).reshape(shape)


def kernel_configs() -> list[str]:
    """Names of the step-kernel configurations, by configuration index."""
    lib = _native.load()
    return [lib.sf_kernel_config_name(q).decode() for q in range(lib.sf_kernel_config_count())]


def has_native_kernels() -> bool:
    """True when a CUDA device is present and the sm_103a library loads."""
    try:
        import torch

        if not torch.cuda.is_available():
            return False
        _native.load()
        return True
    except Exception:
        return False


def has_gpu_backend() -> bool:
    """Whether the reference's PyTorch-MPS backend is available
    (core/solver.py:143-149): never here, where the CUDA kernels are the
    "native" backend and ``backend="gpu"`` is not offered."""
    return False


def get_native_info() -> dict:
    import torch

    info = {"available": has_native_kernels(), "version": None, "device": None}
    if info["available"]:
        info["version"] = _native.load().sf_version().decode()
        info["device"] = torch.cuda.get_device_name()
    return info


class FDTDSolver:
    """3-D acoustic FDTD solver on a staggered grid, stepped on the GPU.

    Arguments as the reference (core/solver.py:1507-1518).  ``backend`` may be
    "auto" or "native"; both select the GB300 kernels.  ``device`` picks the
    CUDA device (default: the current one).
    """

    def __init__(self, shape=None, resolution=None, grid=None, c: float = 343.0,
                 rho: float = 1.2, courant: float = 0.95,
                 backend: Literal["auto", "native"] = "auto", warn_energy_drift: bool = False,
                 energy_drift_threshold: float = 0.01, device=None):
        import torch

        if grid is not None:
            self._grid = grid
            self.shape = tuple(grid.shape)
        elif shape is not None and resolution is not None:
            self._grid = UniformGrid(shape=shape, resolution=resolution)
            self.shape = tuple(self._grid.shape)
        else:
            raise ValueError("Must provide either 'grid' or both 'shape' and 'resolution'")
        if backend not in ("auto", "native"):
            raise ValueError(f"backend must be 'auto' or 'native' (GB300 kernels), got {backend!r}")
        if not torch.cuda.is_available():
            raise RuntimeError("strata_fdtd_gb300 needs a CUDA device; none is available")
        self._lib = _native.load()
        self._torch = torch
        self._device = torch.device("cuda", torch.cuda.current_device() if device is None
                                    else torch.device(device).index or 0)

        self.dx = self._grid.min_spacing
        self.c = c
        self.rho = rho
        self._use_native = True
        self.dt, self._coeff_v, self._coeff_p = step_coefficients(self._grid, c, rho, courant)

        nx, ny, nz = self.shape
        self._n = nx * ny * nz
        with torch.cuda.device(self._device):
            self._dev = [[torch.zeros(self.shape, dtype=torch.float32, device=self._device)
                          for _ in _FIELDS] for _ in range(2)]
        self._host = {f: np.zeros(self.shape, dtype=np.float32) for f in _FIELDS}
        self._host_fresh = {f: True for f in _FIELDS}
        self._host_exposed = {f: False for f in _FIELDS}
        # whether vz was ever handed out or set: until then its last plane
        # (a face no step updates) is known to be zero without a device read
        self._vz_seen = False
        self._geometry = np.ones(self.shape, dtype=bool)
        self._geometry_dev = None
        self._geometry_set = False

        desc = _native.SfGridDesc(nx, ny, nz, float(self._coeff_v), float(self._coeff_p), 0)
        plan = ctypes.c_void_p()
        _native.check(self._lib.sf_plan_create(ctypes.byref(desc), ctypes.byref(plan)),
                      "sf_plan_create")
        self._plan = plan
        ptrs = [t.data_ptr() for s in self._dev for t in s]
        _native.check(self._lib.sf_plan_bind_fields(self._plan, *ptrs), "sf_plan_bind_fields")
        if not self._grid.is_uniform:
            self._set_nonuniform()

        self._sources: list = []
        self._probes: dict[str, Probe] = {}
        self._boundaries: list = []
        self._microphones: dict = {}
        self._src_dirty = True
        self._probe_dirty = True
        self._tables_version = 0  # bumped by every change to geometry, sources, probes, PML, ADE
        self._kernel_auto = True  # no kernel chosen by set_kernel: odd nz may run padded
        self._graph_epoch = 0  # bumped when the plan's kernel choice changes
        self._probe_order: list[str] = []
        self._pending_traces: list = []
        self._mic_order: list = []  # (name, rows) per microphone
        self._mic_rows = 0
        self._mic_dirty = False
        self._pending_mics: list = []

        self._step_count = 0
        self._time = 0.0
        self._snapshots: list = []
        self._velocity_snapshots: list = []
        self._snap_staged: list = []    # (t, device copies, event): waiting for the next steps
        self._snap_inflight: list = []  # (t, futures of the host arrays): copies under way
        self._snap_stream = None
        self._snap_pool = None
        self._snapshot_interval = None
        self._snapshot_velocity = False

        self._warn_energy_drift = warn_energy_drift
        self._energy_drift_threshold = energy_drift_threshold
        self._energy_history: list = []
        self._track_energy = False
        self._energy_sample_interval = 1
        self._energy_scratch = None

        self._materials: dict = {}
        self._material_id = np.zeros(self.shape, dtype=np.uint8)
        self._ade_initialized = False
        self._ade_debye: list = []
        self._ade_lorentz: list = []
        self._mat_dev = None

    def _set_nonuniform(self):
        """Spacing tables of a nonuniform grid (core/solver.py:1587-1602):
        face coefficients float(coeff_v_base) * inv_face in float, as
        update_velocity_nonuniform forms them (fdtd_step.cpp:235-305), and
        the cell inverse spacings of the divergence."""
        sa = self._grid.get_spacing_arrays_for_stencil()
        cvb = np.float32(self._coeff_v)
        face, cell = [], []
        for ax, n in zip("xyz", self.shape):
            f = np.zeros(n, dtype=np.float32)
            f[:n - 1] = cvb * sa[f"inv_d{ax}_face"]
            face.append(f)
            cell.append(np.ascontiguousarray(sa[f"inv_d{ax}_cell"], dtype=np.float32))
        self._nu_tables = face + cell  # kept alive for the copy
        fp = (ctypes.c_void_p * 3)(*[a.ctypes.data for a in face])
        cp = (ctypes.c_void_p * 3)(*[a.ctypes.data for a in cell])
        _native.check(self._lib.sf_plan_set_nonuniform(self._plan, fp, cp), "sf_plan_set_nonuniform")

    def __del__(self):
        pool = getattr(self, "_snap_pool", None)
        if pool is not None:
            pool.shutdown(wait=False)
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                self._lib.sf_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    # ------------------------------------------------------------------ fields
    def _stream(self):
        return self._torch.cuda.current_stream(self._device).cuda_stream

    def _cur(self) -> int:
        return int(self._lib.sf_plan_current(self._plan))

    def _field(self, name):
        if not self._host_fresh[name]:
            src = self._dev[self._cur()][_FIELDS.index(name)]
            self._torch.from_numpy(self._host[name]).copy_(src)
            self._host_fresh[name] = True
        self._host_exposed[name] = True
        self._vz_seen = self._vz_seen or name == "vz"
        return self._host[name]

    def _set_field(self, name, value):
        arr = np.asarray(value)
        if arr.shape != self.shape:
            raise ValueError(f"{name} shape {arr.shape} doesn't match solver shape {self.shape}")
        if not (arr.dtype == np.float32 and arr.flags.c_contiguous and arr.flags.writeable):
            arr = np.ascontiguousarray(arr, dtype=np.float32).copy()
        self._host[name] = arr
        self._host_fresh[name] = True
        self._host_exposed[name] = True
        self._vz_seen = self._vz_seen or name == "vz"

    p = property(lambda s: s._field("p"), lambda s, v: s._set_field("p", v))
    vx = property(lambda s: s._field("vx"), lambda s, v: s._set_field("vx", v))
    vy = property(lambda s: s._field("vy"), lambda s, v: s._set_field("vy", v))
    vz = property(lambda s: s._field("vz"), lambda s, v: s._set_field("vz", v))

    def device_fields(self) -> dict:
        """The current state as CUDA tensors (no copy); valid until the next step."""
        self._vz_seen = True  # the caller may write vz through the tensor
        self._upload_exposed()
        cur = self._cur()
        return {f: self._dev[cur][q] for q, f in enumerate(_FIELDS)}

    def load_fields_async(self, **fields) -> None:
        """Copy host arrays into the device state on the current stream
        without waiting for the copies: any of p, vx, vy, vz, each a
        C-contiguous float32 array of the grid's shape (from pinned memory
        the copies run asynchronously).  The arrays must stay unchanged until
        the copies have run (an event recorded on the stream after this call
        marks that); the fields not given keep their values."""
        torch = self._torch
        for name, value in fields.items():
            if name not in _FIELDS:
                raise ValueError(f"unknown field {name!r}; the fields are {_FIELDS}")
            a = np.asarray(value)
            if a.shape != self.shape or a.dtype != np.float32 or not a.flags.c_contiguous:
                raise ValueError(f"{name} must be a C-contiguous float32 array of shape "
                                 f"{self.shape}")
        self._upload_exposed()
        cur = self._cur()
        for name, value in fields.items():
            self._dev[cur][_FIELDS.index(name)].copy_(torch.from_numpy(np.asarray(value)),
                                                       non_blocking=True)
            self._host_fresh[name] = False
            self._host_exposed[name] = False
            self._vz_seen = self._vz_seen or name == "vz"

    def fields_async(self, names=_FIELDS, out: dict | None = None):
        """Start copying the named fields of the current state to pinned host
        memory, queued on the current stream after the steps so far, and
        return a function that waits for those copies only and returns
        {name: array}.  ``out`` may give a pinned float32 array of the grid's
        shape per name to copy into (no allocation); the arrays must not be
        read before the function returns."""
        torch = self._torch
        self._upload_exposed()
        cur = self._cur()
        dst = {}
        for name in names:
            src = self._dev[cur][_FIELDS.index(name)]
            if out is not None and name in out:
                a = out[name]
                if a.shape != self.shape or a.dtype != np.float32 or not a.flags.c_contiguous:
                    raise ValueError(f"out[{name!r}] must be a C-contiguous float32 array of "
                                     f"shape {self.shape}")
                host = torch.from_numpy(a)
            else:
                host = torch.empty(self.shape, dtype=torch.float32, pin_memory=True)
            host.copy_(src, non_blocking=True)
            dst[name] = host
        done = torch.cuda.Event()
        done.record()

        def result() -> dict:
            done.synchronize()
            return {n: t.numpy() for n, t in dst.items()}

        return result

    def _upload_exposed(self):
        cur = None
        for q, f in enumerate(_FIELDS):
            if self._host_exposed[f]:
                cur = self._cur() if cur is None else cur
                self._dev[cur][q].copy_(self._torch.from_numpy(self._host[f]))
                self._host_exposed[f] = False

    def _mark_device_newer(self):
        for f in _FIELDS:
            self._host_fresh[f] = False

    # --------------------------------------------------------------- geometry
    @property
    def geometry(self) -> np.ndarray:
        return self._geometry

    @geometry.setter
    def geometry(self, mask):
        self.set_geometry(np.asarray(mask))

    @property
    def time(self) -> float:
        return self._time

    @property
    def step_count(self) -> int:
        return self._step_count

    @property
    def using_native(self) -> bool:
        return True

    @property
    def using_gpu(self) -> bool:
        return True

    @property
    def grid(self):
        return self._grid

    def set_geometry(self, geometry) -> None:
        """Boolean mask (True = air), an SDFPrimitive voxelised on the GPU
        with inside = air, or a MaterializedGeometry whose regions also set
        the material ids (core/solver.py:1682-1780)."""
        torch = self._torch
        from .material_assignment import MaterializedGeometry

        if isinstance(geometry, MaterializedGeometry):
            # core/solver.py:1715-1760: the mask, then every non-default
            # material registered under its id (unless already registered)
            # and written where the voxelised ids name it; ids already set
            # elsewhere are left as they are
            dev, mat_dev = geometry.voxelize_with_materials_device(self._grid)
            ids = mat_dev.cpu().numpy()
            self._geometry = dev.cpu().numpy().astype(bool)
            for mid, material in geometry.get_material_table().items():
                if mid == 0:
                    continue
                if mid not in self._materials:
                    self.register_material(material, material_id=mid)
                region = ids == mid
                if region.any():
                    self.set_material_region(region, material_id=mid)
            self._ade_initialized = False
        elif isinstance(geometry, SDFPrimitive):
            dev = geometry.voxelize_device(self._grid)
            self._geometry = dev.cpu().numpy().astype(bool)
            self._material_id.fill(0)
        else:
            mask = np.asarray(geometry)
            if mask.shape != self.shape:
                raise ValueError(f"Geometry shape {mask.shape} doesn't match solver shape {self.shape}")
            self._geometry = mask.astype(bool)
            dev = torch.from_numpy(np.ascontiguousarray(self._geometry).view(np.uint8)).to(
                self._device)
        self._geometry_dev = dev
        self._geometry_set = True
        _native.check(self._lib.sf_plan_set_geometry(self._plan, dev.data_ptr(), self._stream()),
                      "sf_plan_set_geometry")
        self._src_dirty = True  # membrane sources inject into air cells only
        self._tables_version += 1

    def set_geometry_sdf(self, solid: SDFPrimitive) -> None:
        """Geometry from a solid's SDF: air is the complement of the solid
        (``~solid.voxelize(grid)``), voxelised straight into HBM."""
        dev = solid.voxelize_device(self._grid, invert=True)
        self._geometry = dev.cpu().numpy().astype(bool)
        self._geometry_dev = dev
        self._geometry_set = True
        _native.check(self._lib.sf_plan_set_geometry(self._plan, dev.data_ptr(), self._stream()),
                      "sf_plan_set_geometry")
        self._src_dirty = True  # membrane sources inject into air cells only
        self._tables_version += 1

    # --------------------------------------------------------- sources/probes
    def _to_index(self, pos, what):
        if isinstance(pos, tuple) and len(pos) == 3 and any(
                isinstance(p, float) and p < max(self.shape) for p in pos):
            idx = tuple(int(round(p / self.dx)) for p in pos)
            for a, (v, n) in enumerate(zip(idx, self.shape)):
                if not 0 <= v < n:
                    raise ValueError(f"{what} {'xyz'[a]} position {pos[a]:.4f}m "
                                     f"(index {v}) is outside grid (0-{n - 1})")
            return idx
        return pos

    def add_source(self, source) -> None:
        """core/solver.py:1782-1841: point and plane GaussianPulse sources and
        membrane sources (centre inside the physical extent)."""
        if source.source_type == "membrane":
            extent = self._grid.physical_extent()
            for ax, (v, e) in enumerate(zip(source.center, extent)):
                if not 0 <= v <= e:
                    raise ValueError(f"Membrane center {'xyz'[ax]}={v:.4f}m is outside grid "
                                     f"(0-{e:.4f}m)")
        elif source.source_type == "point":
            source.position = self._to_index(source.position, "Source")
            if any(not 0 <= int(v) < n for v, n in zip(source.position, self.shape)):
                raise ValueError(f"Source position {source.position} is outside the grid")
        elif source.source_type == "plane":
            ax, idx = source.position["axis"], source.position["index"]
            if ax not in (0, 1, 2) or not 0 <= idx < self.shape[ax]:
                raise ValueError(f"Plane source {source.position} is outside the grid")
        else:
            raise NotImplementedError(f"source_type {source.source_type!r} is not supported")
        if len(self._sources) >= 16:
            raise ValueError("at most 16 sources are supported")
        self._sources.append(source)
        self._src_cache = None
        self._src_dirty = True
        self._tables_version += 1

    def add_probe(self, name: str, position) -> None:
        """core/solver.py:1843-1885."""
        if name in self._probes:
            raise ValueError(f"Probe '{name}' already exists")
        position = self._to_index(position, "Probe")
        if any(not 0 <= int(v) < n for v, n in zip(position, self.shape)):
            raise ValueError(f"Probe position {position} is outside the grid")
        self._flush_traces()
        self._probes[name] = Probe(name=name, position=tuple(int(v) for v in position),
                                   _solver=self)
        self._probe_dirty = True
        self._tables_version += 1

    def add_microphone(self, position, name=None, pattern="omni", direction=None, up=None):
        """Microphone at a physical position, omnidirectional or with a polar
        pattern (core/solver.py:1887-1965); returns the Microphone."""
        from .microphones import Microphone

        mic = position if isinstance(position, Microphone) else Microphone(
            position=position, name=name, pattern=pattern, direction=direction, up=up)
        mic.name = mic.name or f"mic_{len(self._microphones)}"
        if mic.name in self._microphones:
            raise ValueError(f"Microphone '{mic.name}' already exists")
        mic._initialize(self)
        self._flush_traces()
        self._microphones[mic.name] = mic
        self._mic_dirty = True
        return mic

    @property
    def microphones(self) -> dict:
        return self._microphones

    def add_boundary(self, boundary) -> None:
        """Boundaries act in the order added (core/solver.py:1983-1990,
        2040-2047): the PML inside the fused step, then the pressure-plane
        boundaries (Mur ABC, radiation impedance) in order."""
        if isinstance(boundary, RigidBoundary):
            boundary.initialize(self)
            self._boundaries.append(boundary)
            return
        if isinstance(boundary, (ABCFirstOrder, RadiationImpedance)):
            boundary.initialize(self)
            self._boundaries.append(boundary)
            self._plane_bc_dirty = True
            self._tables_version += 1
            return
        if not isinstance(boundary, PML):
            raise NotImplementedError(f"{type(boundary).__name__} is not supported by the GB300 backend")
        if any(isinstance(b, PML) for b in self._boundaries):
            raise NotImplementedError("one PML per solver is supported by the GB300 backend")
        if any(isinstance(b, (ABCFirstOrder, RadiationImpedance)) for b in self._boundaries):
            raise NotImplementedError("a PML must be added before plane boundaries "
                                      "(the fused step applies it first)")
        boundary.initialize(self)
        self._boundaries.append(boundary)
        sx, sy, sz = boundary.sigmas
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        _native.check(self._lib.sf_plan_set_pml(self._plan, ptr(sx), ptr(sy), ptr(sz),
                                                float(self.dt)), "sf_plan_set_pml")
        self._pml_keepalive = (sx, sy, sz)
        self._tables_version += 1

    def enable_snapshots(self, interval: int, capture_velocity: bool = False) -> None:
        self._snapshot_interval = interval
        self._snapshot_velocity = capture_velocity

    # --------------------------------------------------------------- materials
    def register_material(self, material, material_id: int | None = None) -> int:
        if material_id is None:
            material_id = next((i for i in range(1, 256) if i not in self._materials), None)
            if material_id is None:
                raise ValueError("Maximum of 255 materials reached")
        if not 1 <= material_id <= 255:
            raise ValueError("material_id must be in range 1-255 (0 is reserved for air)")
        if material_id in self._materials:
            raise ValueError(f"Material ID {material_id} is already registered")
        self._materials[material_id] = material
        self._ade_initialized = False
        return material_id

    def set_material_region(self, mask, material_id: int) -> None:
        mask = np.asarray(mask)
        if mask.shape != self.shape:
            raise ValueError(f"Mask shape {mask.shape} doesn't match solver shape {self.shape}")
        if material_id != 0 and material_id not in self._materials:
            raise ValueError(f"Material ID {material_id} not registered. Use register_material() first.")
        self._material_id[mask] = material_id
        self._ade_initialized = False

    def set_material_box(self, material_id, x_range, y_range, z_range) -> None:
        mask = np.zeros(self.shape, dtype=bool)
        mask[x_range[0]:x_range[1], y_range[0]:y_range[1], z_range[0]:z_range[1]] = True
        self.set_material_region(mask, material_id)

    def get_material_at(self, position):
        mid = int(self._material_id[position])
        return None if mid == 0 else self._materials.get(mid)

    @property
    def has_materials(self) -> bool:
        return len(self._materials) > 0

    @property
    def material_count(self) -> int:
        return len(self._materials)

    def _initialize_ade_fields(self) -> None:
        """Pole table and auxiliary fields as _initialize_ade_native
        (core/solver.py:2996-3083): one J per pole, Debye and Lorentz numbered
        separately in registration order; FP32 coefficients formed the way
        ade.cpp forms them (-dt/rho_inf*inv_dx, ade.cpp:263; -K_inf*dt,
        ade.cpp:420)."""
        torch = self._torch
        f32 = np.float32
        dt32 = f32(self.dt)
        inv_dx = f32(1.0 / self.dx)
        debye, lorentz = [], []
        for mid, mat in self._materials.items():
            rho_inf, k_inf = f32(mat.rho_inf), f32(mat.K_inf)
            for pole in mat.poles:
                tgt = 0 if pole.target == "density" else 1
                co = [f32(v) for v in pole.fdtd_coefficients(self.dt)]
                corr = f32(f32(-dt32) / rho_inf) * inv_dx if tgt == 0 else f32(-k_inf) * dt32
                e = dict(mid=mid, target=tgt, co=co, corr=f32(corr),
                         J=torch.zeros(self._n, dtype=torch.float32, device=self._device))
                if pole.is_debye:
                    debye.append(e)
                else:
                    e["Jp"] = torch.zeros(self._n, dtype=torch.float32, device=self._device)
                    lorentz.append(e)
        self._ade_debye, self._ade_lorentz = debye, lorentz
        poles = (_native.SfPole * max(1, len(debye) + len(lorentz)))()
        for q, e in enumerate(debye + lorentz):
            pl = poles[q]
            pl.material_id, pl.kind, pl.target = e["mid"], 0 if "Jp" not in e else 1, e["target"]
            c = list(e["co"]) + [0.0] * (3 - len(e["co"]))
            pl.c0, pl.c1, pl.c2, pl.corr = float(c[0]), float(c[1]), float(c[2]), float(e["corr"])
            pl.J = e["J"].data_ptr()
            pl.J_prev = e["Jp"].data_ptr() if "Jp" in e else None
        n = len(debye) + len(lorentz)
        if n > 16:
            raise NotImplementedError("at most 16 ADE poles are supported")
        self._mat_dev = torch.from_numpy(self._material_id.reshape(-1)).to(self._device)
        _native.check(self._lib.sf_plan_set_ade(self._plan, self._mat_dev.data_ptr(), n,
                                                ctypes.addressof(poles), float(inv_dx)),
                      "sf_plan_set_ade")
        where = np.nonzero(self._material_id)
        lo = [int(w.min()) for w in where] if where[0].size else [0, 0, 0]
        hi = [int(w.max()) + 1 for w in where] if where[0].size else [0, 0, 0]
        _native.check(self._lib.sf_plan_set_ade_box(self._plan, (ctypes.c_int32 * 3)(*lo),
                                                    (ctypes.c_int32 * 3)(*hi)),
                      "sf_plan_set_ade_box")
        self._ade_box = (lo, hi)
        self._ade_inv_dx = inv_dx
        self._ade_initialized = True
        self._tables_version += 1

    @property
    def _ade_J_debye(self) -> np.ndarray:
        parts = [e["J"].cpu().numpy() for e in self._ade_debye]
        return np.concatenate(parts) if parts else np.zeros(1, dtype=np.float32)

    @property
    def _ade_J_lorentz(self) -> np.ndarray:
        parts = [e["J"].cpu().numpy() for e in self._ade_lorentz]
        return np.concatenate(parts) if parts else np.zeros(1, dtype=np.float32)

    @property
    def _ade_J_lorentz_prev(self) -> np.ndarray:
        parts = [e["Jp"].cpu().numpy() for e in self._ade_lorentz]
        return np.concatenate(parts) if parts else np.zeros(1, dtype=np.float32)

    # ---------------------------------------------------------------- stepping
    def _sync_tables(self):
        if getattr(self, "_plane_bc_dirty", False):
            ops = [op for b in self._boundaries if hasattr(b, "plane_ops") for op in b.plane_ops()]
            tab = (_native.SfPlaneBC * max(1, len(ops)))()
            for q, (kind, axis, side, coeff, refl) in enumerate(ops):
                tab[q].kind, tab[q].axis, tab[q].side = kind, axis, side
                tab[q].coeff, tab[q].reflection = coeff, refl
            _native.check(self._lib.sf_plan_set_plane_boundaries(self._plan, len(ops), tab),
                          "sf_plan_set_plane_boundaries")
            self._plane_bc_dirty = False
        if self._src_dirty:
            tab = (_native.SfSource * max(1, len(self._sources)))()
            for q, s in enumerate(self._sources):
                if s.source_type == "point":
                    tab[q].kind, (tab[q].a, tab[q].b, tab[q].c) = 0, tuple(int(v) for v in s.position)
                elif s.source_type == "plane":
                    tab[q].kind, tab[q].a, tab[q].b, tab[q].c = 1, int(s.position["axis"]), int(
                        s.position["index"]), 0
                else:  # membrane: weighted air cells of its plane (core/solver.py:2389-2412)
                    if s._cached_weights is None:
                        s._check_grid_alignment(self._grid)
                        s._cached_weights = s.get_injection_weights(self._grid)
                        s._cached_mask = s._cached_weights > 0
                    cells = np.flatnonzero(s._cached_mask & self._geometry).astype(np.int64)
                    w = np.ascontiguousarray(s._cached_weights.ravel()[cells], dtype=np.float64)
                    _native.check(self._lib.sf_plan_set_weighted_source(
                        self._plan, q, len(cells), cells.ctypes.data, w.ctypes.data),
                        "sf_plan_set_weighted_source")
                    field = 0 if s.injection_type == "pressure" else 1 + "xyz".index(s.normal_axis)
                    tab[q].kind, tab[q].a, tab[q].b, tab[q].c = 2, q, field, 0
            _native.check(self._lib.sf_plan_set_sources(self._plan, len(self._sources),
                                                        ctypes.addressof(tab)), "sf_plan_set_sources")
            self._src_dirty = False
        if self._probe_dirty:
            self._probe_order = list(self._probes)
            cells = np.array([np.ravel_multi_index(self._probes[n].position, self.shape)
                              for n in self._probe_order] or [0], dtype=np.int64)
            _native.check(self._lib.sf_plan_set_probes(self._plan, len(self._probe_order),
                                                       cells.ctypes.data), "sf_plan_set_probes")
            self._probe_dirty = False
        if self._mic_dirty:
            # the reference's Python recording path (FP64 weights) as soon as
            # one microphone is directional, else its native batch kernel
            # (core/solver.py:2441-2461)
            python_path = any(m.is_directional() for m in self._microphones.values())
            self._mic_order = []
            rows = []
            for name, m in self._microphones.items():
                r = m._rows(self.shape, python_path)
                self._mic_order.append((name, len(r)))
                rows.extend(r)
            field = np.array([f for f, _, _ in rows] or [0], dtype=np.int32)
            idx = np.concatenate([c for _, c, _ in rows] or [np.zeros(8, np.int64)])
            w = np.concatenate([x for _, _, x in rows] or [np.zeros(8, np.float32)])
            _native.check(self._lib.sf_plan_set_microphones_ex(
                self._plan, len(rows), field.ctypes.data, idx.ctypes.data, w.ctypes.data),
                "sf_plan_set_microphones")
            self._mic_rows = len(rows)
            self._mic_dirty = False
        if self.has_materials and not self._ade_initialized:
            self._initialize_ade_fields()

    def _source_values(self, n: int) -> np.ndarray:
        """Waveform per step at the FP64-accumulated times (t += dt each
        step, as _time), as _inject_sources evaluates it (core/solver.py:2413)
        one step at a time.  A GaussianPulse is evaluated over all n times in
        one NumPy call: its operations are elementwise, so every value equals
        the one-element call's (the tests check both ways against each other
        and against the reference's values); any other waveform object is
        called one step at a time."""
        vals = np.zeros((n, len(self._sources)), dtype=np.float64)
        if not self._sources:
            return vals
        times = np.empty(n, dtype=np.float64)
        t = self._time
        for q in range(n):
            times[q] = t
            t += self.dt
        for s, src in enumerate(self._sources):
            wf = src.waveform if src.source_type == "membrane" else src
            if type(wf) is GaussianPulse:
                vals[:, s] = wf.waveform(times, self.dt)
            else:
                for q in range(n):
                    vals[q, s] = wf.waveform(np.array([times[q]]), self.dt)[0]
        return vals

    def precompute_sources(self, n: int) -> None:
        """Evaluate the waveform for the next n steps now and keep it on the
        device (a served request does this once at admission)."""
        vals = self._source_values(n)
        self._src_cache = (self._step_count, self._torch.from_numpy(vals).to(self._device))

    def source_table(self, n: int):
        """Device tensor [n, n_sources] of waveform values for the next n
        steps (from the precomputed table when it covers them)."""
        cache = getattr(self, "_src_cache", None)
        if cache is not None:
            start, tab = cache
            off = self._step_count - start
            if 0 <= off and off + n <= tab.shape[0]:
                return tab[off:off + n]
        return self._torch.from_numpy(self._source_values(n)).to(self._device)

    def _padded_twin(self, vz_handed_out: bool):
        """This solve's padded twin (batch.py, _PaddedTwin: z padded to a
        multiple of 4 with solid cells, so the float4 warp tiles run it), made
        once and kept until the tables change, or None when the solve cannot
        use one: nz already a multiple of 4, a nonuniform grid, microphones,
        plane boundaries or membrane sources, offsets past 32 bits, or a
        nonzero last vz plane (checked again when vz was handed out)."""
        nx, ny, nz = self.shape
        if nz % 4 == 0 or not self._grid.is_uniform or self._microphones:
            return None
        if any(hasattr(b, "plane_ops") for b in self._boundaries) or any(
                src.source_type == "membrane" for src in self._sources):
            return None
        nzp = (nz + 3) // 4 * 4
        if nx * ny * nzp + 2 * ny * nzp + 8 >= 2**31 - 1:
            return None
        twin = getattr(self, "_pad_twin", None)
        if twin is not None and (twin.version != self._tables_version or vz_handed_out):
            twin = None
        if twin is None:
            from .batch import _PaddedTwin

            ok = not self._vz_seen or _PaddedTwin.eligible(self)
            twin = _PaddedTwin(self) if ok else None
            self._pad_twin = twin
        return twin

    _TWIN_MIN_STEPS = 32  # runs this long go through the padded twin (two state copies)
    _GRAPH_STEPS = 50     # steps per captured CUDA graph (even: the current set comes back)

    def _graph_for(self, owner, plan, n_src: int, n_probe: int):
        """A CUDA graph of _GRAPH_STEPS steps of ``plan`` from its current
        set, reading the source values of those steps from a device buffer
        and writing their probe rows to another (filled and drained around
        each replay), kept on ``owner`` (this solver or its padded twin) until
        the tables or the kernel choice change.  It replays exactly the
        launches one sf_plan_step call makes, without the host's per-launch
        overhead."""
        torch = self._torch
        cur = int(self._lib.sf_plan_current(plan))
        stamp = (self._tables_version, self._graph_epoch)
        cache = owner.__dict__.setdefault("_graphs", {})
        if cache.get("stamp") != stamp:
            cache.clear()
            cache["stamp"] = stamp
        key = (cur, n_src, n_probe)
        if key in cache:
            return cache[key]
        G = self._GRAPH_STEPS
        src = torch.zeros((G, max(1, n_src)), dtype=torch.float64, device=self._device)
        trace = torch.zeros((G, max(1, n_probe)), dtype=torch.float32, device=self._device)
        stream = torch.cuda.Stream(self._device)
        stream.wait_stream(torch.cuda.current_stream(self._device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            rc = self._lib.sf_plan_step_ex(plan, G, src.data_ptr() if n_src else None,
                                           trace.data_ptr() if n_probe else None, None,
                                           stream.cuda_stream)
        _native.check(rc, "sf_plan_step (graph capture)")
        torch.cuda.current_stream(self._device).wait_stream(stream)
        cache[key] = (g, src, trace)
        return cache[key]

    def _advance(self, n: int) -> None:
        """Run n time steps through one sf_plan_step call."""
        torch = self._torch
        if n <= 0:
            return
        vz_handed_out = self._host_exposed["vz"]
        self._sync_tables()
        self._upload_exposed()
        twin = None
        if n >= self._TWIN_MIN_STEPS and self._kernel_auto:
            twin = self._padded_twin(vz_handed_out)
        src_dev = self.source_table(n) if self._sources else None
        n_probe = len(self._probe_order)
        trace = (torch.empty((n, n_probe), dtype=torch.float32, device=self._device)
                 if n_probe else None)
        n_mic = getattr(self, "_mic_rows", 0)
        mic_trace = (torch.empty((n, n_mic), dtype=torch.float32, device=self._device)
                     if n_mic else None)
        if twin is not None:
            twin.copy_in(self)
        plan = self._plan if twin is None else twin.plan
        G = self._GRAPH_STEPS
        n_graph = 0
        if mic_trace is None and self._kernel_auto and not torch.cuda.is_current_stream_capturing():
            n_graph = n - n % G  # (inside a caller's capture the launches go into its graph)
        if n_graph:
            g, gsrc, gtrace = self._graph_for(twin if twin is not None else self, plan,
                                              len(self._sources), n_probe)
            for q in range(0, n_graph, G):
                if src_dev is not None:
                    gsrc.copy_(src_dev[q:q + G])
                g.replay()
                if trace is not None:
                    trace[q:q + G].copy_(gtrace[:, :n_probe])
        if n > n_graph:
            rc = self._lib.sf_plan_step_ex(
                plan, n - n_graph, None if src_dev is None else src_dev[n_graph:].data_ptr(),
                None if trace is None else trace[n_graph:].data_ptr(),
                None if mic_trace is None else mic_trace.data_ptr(), self._stream())
            _native.check(rc, "sf_plan_step")
        if twin is not None:
            twin.copy_out(self)
        if trace is not None:
            self._pending_traces.append((trace, list(self._probe_order)))
        times = []
        for _ in range(n):
            times.append(self._time)
            self._time += self.dt
        if mic_trace is not None:
            self._pending_mics.append((mic_trace, list(self._mic_order), times))
        self._mark_device_newer()
        self._step_count += n

    def _flush_traces(self):
        for trace, names in self._pending_traces:
            host = trace.cpu().numpy()
            for q, name in enumerate(names):
                if name in self._probes:
                    self._probes[name]._samples.extend(host[:, q].tolist())
        self._pending_traces.clear()
        for trace, layout, times in getattr(self, "_pending_mics", []):
            host = trace.cpu().numpy()
            q = 0
            for name, n_rows in layout:
                if name in self._microphones:
                    self._microphones[name]._append(host[:, q:q + n_rows], times)
                q += n_rows
        self._pending_mics = []

    def step(self) -> None:
        """Advance one time step (core/solver.py:2003-2077)."""
        self._advance(1)
        self._snap_flush()
        self._after_steps(self._step_count - 1, self._step_count)

    def _after_steps(self, first: int, last: int):
        """Snapshots and energy samples for steps first..last-1 (only the
        last of them can be due, run() splits chunks at these points)."""
        s = last - 1
        if self._snapshot_interval and s % self._snapshot_interval == 0:
            self._snap_capture(self._time - self.dt)
        if self._track_energy and last % self._energy_sample_interval == 0:
            self._energy_history.append((last, self._time, self.compute_energy()))

    # ----------------------------------------------------------- snapshots
    # A snapshot (core/solver.py:2050-2068) is staged as device copies on the
    # compute stream.  Once the following steps are queued (_snap_flush) each
    # copy goes to a pinned buffer on a separate stream (pinned blocks are
    # reused through torch's host cache) and a worker thread moves it into
    # the fresh NumPy array the caller receives, so neither the copy nor the
    # host-memory provisioning holds up the steps; get_snapshots() waits.
    _SNAP_MAX_INFLIGHT = 8
    def _snap_capture(self, t: float) -> None:
        torch = self._torch
        f = self.device_fields()
        staged = [f["p"].clone()]
        if self._snapshot_velocity:
            staged += self._centred_velocity_dev(f)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self._device))
        self._snap_staged.append((t, staged, ev))

    def _snap_flush(self) -> None:
        """Issue the device-to-host copies of the staged snapshots."""
        if not self._snap_staged:
            return
        torch = self._torch
        if self._snap_stream is None:
            self._snap_stream = torch.cuda.Stream(self._device)
        if self._snap_pool is None:
            from concurrent.futures import ThreadPoolExecutor
            self._snap_pool = ThreadPoolExecutor(max_workers=4, thread_name_prefix="sf-snapshot")
        for t, staged, ev in self._snap_staged:
            while len(self._snap_inflight) >= self._SNAP_MAX_INFLIGHT:
                self._snap_retire_oldest()
            arrays, futs = [], []
            for x in staged:
                pinned = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
                with torch.cuda.stream(self._snap_stream):
                    self._snap_stream.wait_event(ev)
                    pinned.copy_(x, non_blocking=True)
                    x.record_stream(self._snap_stream)  # kept until the copy is done
                    done = torch.cuda.Event()
                    done.record(self._snap_stream)
                out = _fresh_host_array(tuple(x.shape))
                arrays.append(out)
                n = out.shape[0]
                for q in range(4):  # slabs along x, moved by the workers side by side
                    lo, hi = n * q // 4, n * (q + 1) // 4
                    if hi > lo:
                        futs.append(self._snap_pool.submit(self._snap_slab, pinned, done, out, lo, hi))
            self._snap_inflight.append((t, arrays, futs))
        self._snap_staged.clear()

    @staticmethod
    def _snap_slab(pinned, done, out, lo, hi):
        done.synchronize()
        np.copyto(out[lo:hi], pinned.numpy()[lo:hi])

    def _snap_retire_oldest(self) -> None:
        t, arrays, futs = self._snap_inflight.pop(0)
        for f in futs:
            f.result()
        self._snapshots.append((t, arrays[0]))
        if len(arrays) > 1:
            self._velocity_snapshots.append((t, *arrays[1:]))

    def _snap_collect(self) -> None:
        self._snap_flush()
        while self._snap_inflight:
            self._snap_retire_oldest()

    def _centred_velocity_dev(self, f) -> list:
        """Staggered velocities averaged to cell centres on the device, with
        the reference's float32 operations: c[1:] = 0.5 * (v[:-1] + v[1:]),
        c[0] = 0.5 * v[0] along each velocity's own axis
        (core/solver.py:2647-2687)."""
        out = []
        for ax, name in enumerate(("vx", "vy", "vz")):
            v = f[name]
            n = v.shape[ax]
            c = self._torch.empty_like(v)
            if n > 1:
                c.narrow(ax, 1, n - 1).copy_(0.5 * (v.narrow(ax, 0, n - 1) + v.narrow(ax, 1, n - 1)))
            c.narrow(ax, 0, 1).copy_(0.5 * v.narrow(ax, 0, 1))
            out.append(c)
        return out

    def run(self, duration: float, progress: bool = False, track_energy: bool = False,
            energy_sample_interval: int = 1, output_file: str | None = None,
            script_content: str | None = None, callback=None,
            snapshot_interval: int | None = None) -> None:
        """Advance ceil(duration/dt) steps (core/solver.py:2520-2606)."""
        if output_file:
            raise NotImplementedError("HDF5 output is not implemented by the GB300 backend")
        n_steps = int(np.ceil(duration / self.dt))
        self.run_steps(n_steps, track_energy=track_energy,
                       energy_sample_interval=energy_sample_interval, callback=callback)

    def run_steps(self, n_steps: int, track_energy: bool = False,
                  energy_sample_interval: int = 1, callback=None) -> None:
        """Advance exactly n_steps, in as few C-ABI calls as the snapshot,
        energy and callback settings allow."""
        self._track_energy = track_energy
        self._energy_sample_interval = energy_sample_interval
        if track_energy and not self._energy_history:
            self._energy_history.append((self._step_count, self._time, self.compute_energy()))
        done = 0
        while done < n_steps:
            chunk = min(n_steps - done, _MAX_CHUNK)
            if callback is not None:
                chunk = 1
            if self._snapshot_interval:
                iv = self._snapshot_interval
                nxt = ((self._step_count + iv - 1) // iv) * iv  # next due pre-increment index
                chunk = min(chunk, nxt - self._step_count + 1)
            if track_energy:
                iv = energy_sample_interval
                nxt = ((self._step_count // iv) + 1) * iv
                chunk = min(chunk, nxt - self._step_count)
            first = self._step_count
            self._advance(chunk)
            self._snap_flush()  # copies of the previous snapshot run beside this chunk
            self._after_steps(first, self._step_count)
            if callback is not None:
                callback(self._step_count - 1)
            done += chunk
        self._snap_flush()
        if self._warn_energy_drift and len(self._energy_history) >= 2:
            rep = self.energy_report()
            if abs(rep["energy_change_percent"]) > self._energy_drift_threshold * 100:
                warnings.warn(f"Energy drift detected: {rep['energy_change_percent']:.2f}% change",
                              UserWarning, stacklevel=2)

    def set_kernel(self, variant: str = "auto", i_chunk: int = 0) -> None:
        """Choose the step kernel by name: "auto", "cell" (one thread per
        cell), "march" (2.5-D slab march with shared-memory halos), "col"
        (thread columns along i, float4 along k when nz % 4 == 0), "col1"
        (scalar columns) or any name from :func:`kernel_configs`;
        ``i_chunk`` planes per block (0 = automatic).  ADE materials always
        use "cell".  Results are identical."""
        names = kernel_configs()
        name = "col4" if variant == "col" else variant
        if name not in names:
            raise ValueError(f"unknown kernel {variant!r}; choose from {names}")
        _native.check(self._lib.sf_plan_set_kernel(self._plan, names.index(name), int(i_chunk)),
                      "sf_plan_set_kernel")
        self._kernel_auto = name == "auto" and int(i_chunk) == 0
        self._graph_epoch += 1

    def autotune(self, launches: int = 20) -> dict:
        """Time every kernel configuration on this grid (the state is left
        unchanged) and make the fastest the automatic choice.  Returns
        {name: ms per step} and the chosen name under "best"."""
        import ctypes as C

        self._sync_tables()
        self._upload_exposed()
        names = kernel_configs()
        ms = (C.c_float * len(names))()
        best = C.c_int()
        _native.check(self._lib.sf_plan_autotune(self._plan, int(launches), self._stream(),
                                                 ms, C.byref(best)), "sf_plan_autotune")
        self._graph_epoch += 1
        out = {n: float(ms[q]) for q, n in enumerate(names) if ms[q] >= 0}
        out["best"] = names[best.value]
        return out

    def synchronize(self) -> None:
        self._torch.cuda.synchronize(self._device)

    # ----------------------------------------------------------------- outputs
    def probe_data_async(self):
        """Start copying every probe trace still on the device to pinned host
        memory, queued on the current stream after the steps so far, and
        return a function that waits for those copies only (not for work
        queued later on the stream) and returns get_probe_data()'s dict."""
        torch = self._torch
        copies = []
        stream = torch.cuda.current_stream(self._device)
        for trace, names in self._pending_traces:
            host = torch.empty(trace.shape, dtype=trace.dtype, pin_memory=True)
            host.copy_(trace, non_blocking=True)
            # the trace may have been allocated on another stream: keep its
            # block from reuse until this stream's copy has run
            trace.record_stream(stream)
            copies.append((host, names))
        self._pending_traces = []
        done = torch.cuda.Event()
        done.record()

        def result() -> dict:
            done.synchronize()
            for host, names in copies:
                arr = host.numpy()
                for q, name in enumerate(names):
                    if name in self._probes:
                        self._probes[name]._samples.extend(arr[:, q].tolist())
            copies.clear()
            return {n: np.array(pr._samples, dtype=np.float32) for n, pr in self._probes.items()}

        return result

    def get_probe_data(self, name: str | None = None) -> dict:
        self._flush_traces()
        if name is not None:
            if name not in self._probes:
                raise KeyError(f"Probe '{name}' not found")
            return {name: self._probes[name].get_data()}
        return {n: pr.get_data() for n, pr in self._probes.items()}

    def get_snapshots(self):
        self._snap_collect()
        return self._snapshots

    def get_velocity_snapshots(self):
        self._snap_collect()
        return self._velocity_snapshots

    def compute_energy(self) -> float:
        """(1/2)(p^2/(rho c^2) + rho |v|^2) dV summed over air cells, reduced
        in FP64 on the GPU (core/solver.py:2689-2705 sums in FP32)."""
        torch = self._torch
        self._upload_exposed()
        need = int(self._lib.sf_energy_scratch_doubles(self._plan))
        if self._energy_scratch is None or self._energy_scratch.numel() < need:
            self._energy_scratch = torch.empty(need, dtype=torch.float64, device=self._device)
        out = ctypes.c_double()  # without a geometry every cell counts as air
        _native.check(self._lib.sf_plan_energy(self._plan, float(self.rho), float(self.c),
                                               float(self.dx), self._energy_scratch.data_ptr(),
                                               ctypes.byref(out), self._stream()), "sf_plan_energy")
        return float(out.value)

    def get_energy_history(self):
        return self._energy_history.copy()

    def energy_report(self) -> dict:
        if not self._energy_history:
            raise ValueError("No energy history recorded. Call run() with track_energy=True first.")
        e = np.array([v for _, _, v in self._energy_history])
        e0, e1 = e[0], e[-1]
        change = (0.0 if e1 == 0 else float("inf")) if e0 == 0 else (e1 - e0) / e0 * 100
        status = "stable" if abs(change) <= 1.0 else ("growing" if change > 0 else "decaying")
        return {"initial_energy": float(e0), "final_energy": float(e1),
                "max_energy": float(e.max()), "min_energy": float(e.min()),
                "energy_change_percent": change, "conservation_status": status,
                "n_samples": len(e)}

    def reset(self) -> None:
        """core/solver.py:2781-2800."""
        for s in self._dev:
            for t in s:
                t.zero_()
        for f in _FIELDS:
            self._host[f].fill(0)
            self._host_fresh[f] = True
            self._host_exposed[f] = False
        self._step_count = 0
        self._time = 0.0
        self._src_cache = None
        self._snap_collect()
        self._snapshots.clear()
        self._energy_history.clear()
        self._track_energy = False
        self._pending_traces.clear()
        self._pending_mics = []
        for pr in self._probes.values():
            pr._samples.clear()
        for m in self._microphones.values():
            m._data.clear()
            m._times.clear()
        for b in self._boundaries:
            b.reset()
        for e in self._ade_debye + self._ade_lorentz:
            e["J"].zero_()
            if "Jp" in e:
                e["Jp"].zero_()

    def get_sample_rate(self) -> float:
        return 1.0 / self.dt

    def get_frequency_response(self, probe_name: str, n_fft: int | None = None):
        data = self.get_probe_data(probe_name)[probe_name]
        if n_fft is None:
            n_fft = int(2 ** np.ceil(np.log2(len(data))))
        spectrum = np.fft.rfft(data, n=n_fft)
        return np.fft.rfftfreq(n_fft, self.dt), np.abs(spectrum)


__all__ = ["FDTDSolver", "GaussianPulse", "Probe", "has_native_kernels", "get_native_info",
           "has_gpu_backend"]
