"""Differentiable solve: probe-trace loss w.r.t. a per-cell density field.

The forward model is the reference's staggered update (core/solver.py
step order, PML decays, point GaussianPulse source, probes) with a per-cell
density rho = rho0 * (1 + theta); every face velocity uses
cv = -(dt/dx) (1/rho_lo + 1/rho_hi) / 2 while the bulk modulus K = rho0 c^2
stays fixed.  The reference has a scalar density only
(core/solver.py:1584-1586): the design field theta is an extension.

Gradients come from hand-written reverse-time adjoint kernels
(``sf_diff_*``, strata_fdtd_gb300/csrc/sf_adjoint.cu) behind a
``torch.autograd.Function``.  The forward keeps a state checkpoint every K
steps; the backward recomputes each K-step segment from its checkpoint
(storing that segment's pressures) and runs the adjoint back through it, so
memory is O(N * (steps/K + K)) instead of O(N * steps).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .boundaries import PML
from .grid import UniformGrid
from .solver import GaussianPulse, step_coefficients


class _Desc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("dtype", ctypes.c_int32), ("cp", ctypes.c_double), ("dt_over_dx", ctypes.c_double),
                ("rho0", ctypes.c_double), ("decay", ctypes.c_void_p * 3),
                ("src_cell", ctypes.c_int64), ("n_probe", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("probe_cells", ctypes.c_void_p),
                ("geometry", ctypes.c_void_p), ("occupancy", ctypes.c_void_p),
                ("unit_lo", ctypes.c_int32 * 3), ("unit_hi", ctypes.c_int32 * 3)]


def _unit_range(decay: np.ndarray) -> tuple:
    """[lo, hi): the longest run of indices whose decay is exactly 1 along
    with both neighbours' (an index past either end counts as 1)."""
    one = np.concatenate([[True], decay == 1.0, [True]])
    ok = one[:-2] & one[1:-1] & one[2:]
    best, start = (0, 0), None
    for i, v in enumerate(np.append(ok, False)):
        if v and start is None:
            start = i
        elif not v and start is not None:
            if i - start > best[1] - best[0]:
                best = (start, i)
            start = None
    return best


def _ptrs(ts):
    arr = (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])
    return arr


class DifferentiableSolver:
    """A fixed acoustic setup whose probe traces are differentiated w.r.t. a
    density-scale field ``theta`` (shape = grid shape, values >= 0).

    ``dtype`` is the working precision of the forward and adjoint states:
    "dw" (default) double-word floats -- each value the unevaluated sum of
    two floats, about 48 bits, computed on the FP32 pipe (GB300 runs FP64
    at a small fraction of its FP32 rate) --, torch.float64, or
    torch.float32 (fastest, about 1e-3 worst-cell relative gradient error
    after 2000 steps).  Design fields, traces and gradients are float64 for
    "dw" and the working dtype otherwise.

    ``geometry`` (optional, grid shape, True = air, as the reference's
    ``set_geometry``) adds rigid walls: every face that touches a solid cell
    keeps zero velocity and solid cells zero pressure, the reference's rigid
    boundary for a solve started from rest.  The gradient is then taken with
    respect to theta in the air cells (zero in solid ones, whose density
    never enters the solve); a source in a solid cell injects nothing, as in
    the reference.

    An occupancy field ``phi`` (grid shape, values in [0, 1], the solid
    fraction of each cell) can be passed with theta to ``forward`` and
    ``loss``: every face coefficient is scaled by the open fractions of its
    two cells, (1 - phi_lo)(1 - phi_hi), so phi = 1 is a rigid wall and the
    loss is differentiable in the geometry as well as in the density; with a
    phi that requires grad, ``loss(...).backward()`` fills both gradients."""

    def __init__(self, shape, resolution=1e-3, c=343.0, rho0=1.204, courant=0.5, pml_depth=10,
                 source=None, frequency=1500.0, probes=(), dtype="dw", checkpoint_every=100,
                 geometry=None):
        import torch

        self.torch = torch
        if dtype is None or dtype == "dw":
            self.precision = "dw"
            self.dtype = torch.float64      # storage: 8 bytes per value (hi, lo floats)
            self.ext_dtype = torch.float64  # design field, traces, gradients
        elif dtype in (torch.float32, torch.float64):
            self.precision = "f32" if dtype == torch.float32 else "f64"
            self.dtype = self.ext_dtype = dtype
        else:
            raise ValueError("dtype must be 'dw', torch.float32 or torch.float64")
        self.grid = UniformGrid(shape, resolution)
        self.shape = tuple(self.grid.shape)
        self.n = int(np.prod(self.shape))
        self.c, self.rho0 = c, rho0
        self.dt, _, _ = step_coefficients(self.grid, c, rho0, courant)
        self.dx = self.grid.min_spacing
        self.cp = -rho0 * c**2 * self.dt / self.dx  # core/solver.py:1585 with rho0
        self.K = int(checkpoint_every)
        dev = torch.device("cuda")
        self.dev = dev
        # PML decays exp(-sigma dt) in the working precision, from the
        # reference's sigma profile evaluated in double
        pml = PML(depth=pml_depth)

        class _S:
            pass

        stub = _S()
        stub.shape, stub.c, stub.grid = self.shape, c, self.grid
        pml.initialize(stub)
        self.decay, self._unit = [], []
        for n in self.shape:
            d = np.exp(-pml._create_profile(n, np.float64) * self.dt)
            self.decay.append(self._working(d))
            self._unit.append(_unit_range(d))
        self.source = tuple(source) if source is not None else tuple(n // 2 for n in self.shape)
        self.pulse = GaussianPulse(position=self.source, frequency=frequency)
        self.probe_pos = [tuple(p) for p in probes]
        cells = [int(np.ravel_multi_index(p, self.shape)) for p in self.probe_pos]
        self.probe_cells = torch.tensor(cells or [0], dtype=torch.int64, device=dev)
        self.geometry = None
        self._air = None
        if geometry is not None:
            g = np.asarray(geometry, dtype=bool)
            if g.shape != self.shape:
                raise ValueError(f"geometry shape {g.shape} does not match the grid {self.shape}")
            self.geometry = g
            self._air = torch.from_numpy(g.astype(np.uint8)).to(dev)
        self.lib = _native.load()

    def _working(self, values):
        """A device tensor of FP64 values in the working precision (for "dw"
        each value as its nearest (hi, lo) float pair, packed in 8 bytes)."""
        torch = self.torch
        v = np.ascontiguousarray(values, dtype=np.float64)
        if self.precision != "dw":
            return torch.tensor(v, dtype=self.dtype, device=self.dev)
        pair = np.empty(v.shape + (2,), dtype=np.float32)
        pair[..., 0] = v.astype(np.float32)
        pair[..., 1] = (v - pair[..., 0].astype(np.float64)).astype(np.float32)
        return torch.from_numpy(pair.view(np.float64).reshape(v.shape).copy()).to(self.dev)

    def _desc(self, occupancy=None):
        d = _Desc()
        d.nx, d.ny, d.nz = self.shape
        d.dtype = {"f32": 0, "f64": 1, "dw": 2}[self.precision]
        d.cp = self.cp
        d.dt_over_dx = self.dt / self.dx
        d.rho0 = self.rho0
        for a in range(3):
            d.decay[a] = self.decay[a].data_ptr()
        d.src_cell = int(np.ravel_multi_index(self.source, self.shape))
        if self.geometry is not None and not self.geometry[self.source]:
            d.src_cell = -1  # the reference injects into air cells only
        d.n_probe = len(self.probe_pos)
        d.probe_cells = self.probe_cells.data_ptr()
        d.geometry = self._air.data_ptr() if self._air is not None else None
        d.occupancy = occupancy.data_ptr() if occupancy is not None else None
        for a in range(3):
            d.unit_lo[a], d.unit_hi[a] = self._unit[a]
        return d

    def _occupancy(self, occupancy):
        if occupancy is None:
            return None
        occ = occupancy.detach().to(device=self.dev, dtype=self.ext_dtype).contiguous()
        if tuple(occ.shape) != self.shape:
            raise ValueError(f"occupancy shape {tuple(occ.shape)} does not match the grid "
                             f"{self.shape}")
        return occ

    def source_values(self, n_steps):
        """Pulse value per step at the FP64-accumulated times t += dt, in one
        NumPy call over all times (the pulse's operations are elementwise, so
        each value equals the one-time call's)."""
        times = np.empty(n_steps, dtype=np.float64)
        t = 0.0
        for q in range(n_steps):
            times[q] = t
            t += self.dt
        vals = self.pulse.waveform(times, self.dt)
        return self.torch.tensor(vals, dtype=self.ext_dtype, device=self.dev)

    def _source_table(self, n_steps):
        """The source values in the working type, as the forward kernel adds
        them (a double-word solve gets each value's nearest (hi, lo) pair)."""
        if self.precision != "dw":
            return self.source_values(n_steps)
        return self._working(self.source_values(n_steps).cpu().numpy())

    def _stream(self):
        return self.torch.cuda.current_stream().cuda_stream

    def coefficients(self, theta, occupancy=None):
        torch = self.torch
        occ = self._occupancy(occupancy)
        cv = [torch.empty(self.shape, dtype=self.dtype, device=self.dev) for _ in range(3)]
        _native.check(self.lib.sf_diff_coefficients(ctypes.byref(self._desc(occ)), theta.data_ptr(),
                                                    *[c.data_ptr() for c in cv], self._stream()),
                      "sf_diff_coefficients")
        return cv

    def _zeros4(self):
        return [self.torch.zeros(self.shape, dtype=self.dtype, device=self.dev) for _ in range(4)]

    def forward(self, theta, n_steps, keep_checkpoints=True, occupancy=None):
        """Run n_steps from rest.  Returns (trace [n, n_probe], checkpoints,
        face coefficients, source values)."""
        torch = self.torch
        theta = theta.to(self.ext_dtype).contiguous()
        cv = self.coefficients(theta, occupancy)
        sets = [self._zeros4(), self._zeros4()]
        cur = 0
        src = self._source_table(n_steps)
        trace = torch.zeros((n_steps, max(1, len(self.probe_pos))), dtype=self.ext_dtype,
                            device=self.dev)
        ckpts = []
        desc = self._desc()
        for s0 in range(0, n_steps, self.K):
            n = min(self.K, n_steps - s0)
            if keep_checkpoints:
                ckpts.append([t.clone() for t in sets[cur]])
            _native.check(self.lib.sf_diff_forward(
                ctypes.byref(desc), _ptrs(cv), _ptrs(sets[0]), _ptrs(sets[1]), cur, n,
                src[s0:].data_ptr(), trace[s0:].data_ptr(), None, self._stream()),
                "sf_diff_forward")
            cur = (cur + n) & 1
        return trace[:, :len(self.probe_pos)], ckpts, cv, src

    def gradient(self, theta, trace, target, ckpts, cv, src, weight=1.0, occupancy=None):
        """dL/dtheta of L = weight * sum((trace - target)^2) by checkpointed
        recomputation and the reverse-time adjoint; with an occupancy field,
        (dL/dtheta, dL/dphi)."""
        torch = self.torch
        n_steps = trace.shape[0]
        theta = theta.to(self.ext_dtype).contiguous()
        full = torch.zeros((n_steps, max(1, len(self.probe_pos))), dtype=self.ext_dtype,
                           device=self.dev)
        full[:, :trace.shape[1]] = trace
        tgt = torch.zeros_like(full)
        tgt[:, :target.shape[1]] = target.to(self.ext_dtype)
        lam = [self._zeros4(), self._zeros4()]
        lcur = 0
        # per-face dL/dcv sums run over every step: 8 bytes per face (a double,
        # or for an FP32 or double-word solve a double-word float pair), zero-filled
        grad_cv = [torch.zeros(self.shape, dtype=torch.float64, device=self.dev) for _ in range(3)]
        desc = self._desc()
        store = torch.empty((self.K,) + self.shape, dtype=self.dtype, device=self.dev)
        seg_starts = list(range(0, n_steps, self.K))
        for si in reversed(range(len(seg_starts))):
            s0 = seg_starts[si]
            n = min(self.K, n_steps - s0)
            work = [[t.clone() for t in ckpts[si]], self._zeros4()]
            _native.check(self.lib.sf_diff_forward(
                ctypes.byref(desc), _ptrs(cv), _ptrs(work[0]), _ptrs(work[1]), 0, n,
                src[s0:].data_ptr(), None, store.data_ptr(), self._stream()), "sf_diff_forward")
            _native.check(self.lib.sf_diff_adjoint(
                ctypes.byref(desc), _ptrs(cv), _ptrs(lam[0]), _ptrs(lam[1]), lcur, n,
                store.data_ptr(), full[s0:].data_ptr(), tgt[s0:].data_ptr(), float(weight),
                _ptrs(grad_cv), self._stream()), "sf_diff_adjoint")
            lcur = (lcur + n) & 1
        occ = self._occupancy(occupancy)
        out = torch.empty(self.shape, dtype=self.ext_dtype, device=self.dev)
        out_occ = None if occ is None else torch.empty_like(out)
        _native.check(self.lib.sf_diff_grad_fields(
            ctypes.byref(self._desc(occ)), theta.data_ptr(), _ptrs(grad_cv), out.data_ptr(),
            None if out_occ is None else out_occ.data_ptr(), self._stream()), "sf_diff_grad_fields")
        return out if occ is None else (out, out_occ)

    def loss(self, theta, target, n_steps, occupancy=None):
        """L2 loss of the probe traces against ``target`` [n_steps, n_probe],
        differentiable w.r.t. ``theta`` (and ``occupancy``, when given)
        through the adjoint kernels."""
        return ProbeLoss.apply(theta, target, self, n_steps, occupancy)


def _make_function():
    import torch

    class ProbeLossFn(torch.autograd.Function):
        """loss = sum((trace(theta) - target)^2); backward via the adjoint."""

        @staticmethod
        def forward(ctx, theta, target, solver, n_steps, occupancy=None):
            occ = None if occupancy is None else occupancy.detach()
            trace, ckpts, cv, src = solver.forward(theta.detach(), n_steps, occupancy=occ)
            loss = ((trace - target.to(trace.dtype)) ** 2).sum()
            ctx.solver = solver
            ctx.saved = (trace, ckpts, cv, src)
            ctx.save_for_backward(theta, target, occupancy)
            return loss.to(theta.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            theta, target, occupancy = ctx.saved_tensors
            trace, ckpts, cv, src = ctx.saved
            g = ctx.solver.gradient(theta.detach(), trace, target, ckpts, cv, src,
                                    weight=float(grad_out),
                                    occupancy=None if occupancy is None else occupancy.detach())
            if occupancy is None:
                return g.to(theta.dtype), None, None, None, None
            return g[0].to(theta.dtype), None, None, None, g[1].to(occupancy.dtype)

    return ProbeLossFn


class _Lazy:
    fn = None

    @classmethod
    def apply(cls, *a):
        if cls.fn is None:
            cls.fn = _make_function()
        return cls.fn.apply(*a)


ProbeLoss = _Lazy


def reference_loss_torch(solver: DifferentiableSolver, theta, target, n_steps, occupancy=None):
    """The same scheme stepped with plain PyTorch tensor ops (for checking the
    adjoint kernels with torch.autograd at small sizes).  Not used by the
    GPU path."""
    torch = solver.torch
    dt_dx, rho0 = solver.dt / solver.dx, solver.rho0
    rho = rho0 * (1 + theta)
    b = 1.0 / rho
    cvx = -dt_dx * 0.5 * (b[:-1] + b[1:])
    cvy = -dt_dx * 0.5 * (b[:, :-1] + b[:, 1:])
    cvz = -dt_dx * 0.5 * (b[:, :, :-1] + b[:, :, 1:])
    if occupancy is not None:
        w = 1.0 - occupancy
        cvx = cvx * (w[:-1] * w[1:])
        cvy = cvy * (w[:, :-1] * w[:, 1:])
        cvz = cvz * (w[:, :, :-1] * w[:, :, 1:])
    inject = True
    if solver.geometry is not None:
        air = torch.as_tensor(solver.geometry, device=theta.device).to(theta.dtype)
        cvx = cvx * (air[:-1] * air[1:])
        cvy = cvy * (air[:, :-1] * air[:, 1:])
        cvz = cvz * (air[:, :, :-1] * air[:, :, 1:])
        inject = bool(solver.geometry[solver.source])
    dx, dy, dz = solver.decay
    p = torch.zeros_like(theta)
    vx, vy, vz = torch.zeros_like(theta), torch.zeros_like(theta), torch.zeros_like(theta)
    src = solver.source_values(n_steps).to(theta.dtype)
    si, sj, sk = solver.source
    traces = []
    for n in range(n_steps):
        vx = torch.cat([vx[:-1] + cvx * (p[1:] - p[:-1]), vx[-1:]], 0)
        vy = torch.cat([vy[:, :-1] + cvy * (p[:, 1:] - p[:, :-1]), vy[:, -1:]], 1)
        vz = torch.cat([vz[:, :, :-1] + cvz * (p[:, :, 1:] - p[:, :, :-1]), vz[:, :, -1:]], 2)
        div = (vx - torch.nn.functional.pad(vx, (0, 0, 0, 0, 1, 0))[:-1]
               + vy - torch.nn.functional.pad(vy, (0, 0, 1, 0))[:, :-1]
               + vz - torch.nn.functional.pad(vz, (1, 0))[:, :, :-1])
        p = p + solver.cp * div
        vx = vx * dx[:, None, None]
        vy = vy * dy[None, :, None]
        vz = vz * dz[None, None, :]
        p = p * dx[:, None, None] * dy[None, :, None] * dz[None, None, :]
        onehot = torch.zeros_like(p)
        onehot[si, sj, sk] = 1.0 if inject else 0.0
        p = p + src[n] * onehot
        traces.append(torch.stack([p[q] for q in solver.probe_pos]))
    trace = torch.stack(traces)
    return ((trace - target) ** 2).sum()
