"""Batched solves: many FDTDSolver instances stepped together on one GPU.

Each member is an ordinary, fully configured :class:`FDTDSolver` (grid size,
geometry, PML, sources, probes, microphones, nonuniform spacing and ADE
materials may all differ).  A run issues, per time step, one persistent
launch whose blocks pull (grid, i-chunk, rows, columns) tiles from a device
work queue (``sf_batch_*`` in include/sf_gb300.h), then one launch that
samples every member's probes and microphone rows; members with fewer steps
drop out when they are done.  Members with plane boundaries (Mur ABC,
radiation impedance) or membrane sources need ordered per-plane passes
after each step, and a nonuniform grid with ADE materials needs the
per-cell nonuniform ADE kernel: those step through their own single-grid
plan within the same run.  Every member's fields, traces, microphone
waveforms and auxiliary ADE fields are bit-identical to running it alone.
No counterpart in the reference, which steps one solver at a time.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


PLAIN_KERNELS = ("column", "warp", "warp_prefetch", "warp_prefetch_m8")


class _PaddedTwin:
    """A member whose nz is not a multiple of 4, re-planned with z padded to
    the next multiple of 4 so the batch runs float4 warp tiles on it (scalar
    tiles cost about half again as much per cell).  The padding cells are
    solid: flag byte 0, so they are never updated or injected into and hold
    zero pressure and velocity, and the face between the last real plane
    and the padding is held at zero like every face into a solid.  The
    reference never updates that face (the last plane of vz), so it stays at
    its value, which is zero unless set by hand: a member whose last vz plane
    is nonzero is batched as it is.  The PML decays of the padding are 1,
    probe cells are re-indexed, ADE material ids and auxiliary fields are
    padded copies.  State goes into the twin before a run and back after it;
    the cells are the member's cells, so results are bit-identical."""

    def __init__(self, s):
        from .boundaries import PML

        torch, lib = s._torch, s._lib
        nx, ny, nz = s.shape
        self.nz, self.nzp = nz, (nz + 3) // 4 * 4
        shp = (nx, ny, self.nzp)
        dev = s._device
        self.version = s._tables_version
        self.f = [[torch.zeros(shp, dtype=torch.float32, device=dev) for _ in range(4)]
                  for _ in range(2)]
        desc = _native.SfGridDesc(nx, ny, self.nzp, float(s._coeff_v), float(s._coeff_p), 0)
        plan = ctypes.c_void_p()
        _native.check(lib.sf_plan_create(ctypes.byref(desc), ctypes.byref(plan)), "sf_plan_create")
        self.plan, self._lib = plan, lib
        _native.check(lib.sf_plan_bind_fields(plan, *[t.data_ptr() for st in self.f for t in st]),
                      "sf_plan_bind_fields")
        stream = torch.cuda.current_stream(dev).cuda_stream
        geom = torch.zeros(shp, dtype=torch.uint8, device=dev)
        geom[..., :nz] = torch.from_numpy(np.ascontiguousarray(s._geometry).view(np.uint8)).to(dev)
        self._geom = geom
        _native.check(lib.sf_plan_set_geometry(plan, geom.data_ptr(), stream), "sf_plan_set_geometry")
        pml = [b for b in s._boundaries if isinstance(b, PML)]
        if pml:
            sx, sy, sz = pml[0].sigmas
            if sz is not None:
                sz = np.ascontiguousarray(np.concatenate([sz, np.zeros(self.nzp - nz, sz.dtype)]),
                                          dtype=np.float32)
            self._pml = (sx, sy, sz)
            ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
            _native.check(lib.sf_plan_set_pml(plan, ptr(sx), ptr(sy), ptr(sz), float(s.dt)),
                          "sf_plan_set_pml")
        tab = (_native.SfSource * max(1, len(s._sources)))()
        for q, src in enumerate(s._sources):
            if src.source_type == "point":
                tab[q].kind, (tab[q].a, tab[q].b, tab[q].c) = 0, tuple(int(v) for v in src.position)
            else:
                tab[q].kind, tab[q].a, tab[q].b = 1, int(src.position["axis"]), int(src.position["index"])
        _native.check(lib.sf_plan_set_sources(plan, len(s._sources), ctypes.addressof(tab)),
                      "sf_plan_set_sources")
        cells = np.array([np.ravel_multi_index(s._probes[n].position, shp) for n in s._probe_order]
                         or [0], dtype=np.int64)
        _native.check(lib.sf_plan_set_probes(plan, len(s._probe_order), cells.ctypes.data),
                      "sf_plan_set_probes")
        self.J = []
        if s.has_materials:
            entries = s._ade_debye + s._ade_lorentz
            poles = (_native.SfPole * max(1, len(entries)))()
            for q, e in enumerate(entries):
                J = torch.zeros(shp, dtype=torch.float32, device=dev)
                Jp = torch.zeros(shp, dtype=torch.float32, device=dev) if "Jp" in e else None
                self.J.append((e, J, Jp))
                pl = poles[q]
                pl.material_id, pl.kind, pl.target = e["mid"], 0 if Jp is None else 1, e["target"]
                c = list(e["co"]) + [0.0] * (3 - len(e["co"]))
                pl.c0, pl.c1, pl.c2, pl.corr = float(c[0]), float(c[1]), float(c[2]), float(e["corr"])
                pl.J = J.data_ptr()
                pl.J_prev = None if Jp is None else Jp.data_ptr()
            mat = torch.zeros(shp, dtype=torch.uint8, device=dev)
            mat[..., :nz] = s._mat_dev.view(nx, ny, nz)
            self._mat = mat
            _native.check(lib.sf_plan_set_ade(plan, mat.data_ptr(), len(entries),
                                              ctypes.addressof(poles), float(s._ade_inv_dx)),
                          "sf_plan_set_ade")
            lo, hi = s._ade_box
            _native.check(lib.sf_plan_set_ade_box(plan, (ctypes.c_int32 * 3)(*lo),
                                                  (ctypes.c_int32 * 3)(*hi)), "sf_plan_set_ade_box")

    @staticmethod
    def eligible(s) -> bool:
        """The member's last vz plane is zero (the face the padding holds at zero)."""
        nz = s.shape[2]
        return float(s._dev[s._cur()][3][..., nz - 1].abs().max()) == 0.0

    def copy_in(self, s):
        cur, nz = s._cur(), self.nz
        for q in range(4):
            self.f[cur][q][..., :nz].copy_(s._dev[cur][q])
        for e, J, Jp in self.J:
            J[..., :nz].copy_(e["J"].view(J.shape[0], J.shape[1], nz))
            if Jp is not None:
                Jp[..., :nz].copy_(e["Jp"].view(J.shape[0], J.shape[1], nz))
        _native.check(self._lib.sf_plan_set_current(self.plan, cur), "sf_plan_set_current")

    def copy_out(self, s):
        cur, nz = int(self._lib.sf_plan_current(self.plan)), self.nz
        for q in range(4):
            s._dev[cur][q].copy_(self.f[cur][q][..., :nz])
        for e, J, Jp in self.J:
            e["J"].view(J.shape[0], J.shape[1], nz).copy_(J[..., :nz])
            if Jp is not None:
                e["Jp"].view(J.shape[0], J.shape[1], nz).copy_(Jp[..., :nz])
        _native.check(self._lib.sf_plan_set_current(s._plan, cur), "sf_plan_set_current")

    def __del__(self):
        plan = getattr(self, "plan", None)
        if plan is not None and plan.value:
            try:
                self._lib.sf_plan_destroy(plan)
            except Exception:
                pass
            self.plan = None


class BatchedSolver:
    """Steps ``solvers`` together.  ``rows`` (4, 8, 16) and ``i_chunk``
    (planes per tile, 0 = 16) set the tile shape and ``kernel`` (one of
    PLAIN_KERNELS) the kernel of the tiles away from material boxes;
    :meth:`autotune` picks all three."""

    PAD_MIN_CELLS = 1 << 25  # total cells of a run from which members are padded

    def __init__(self, solvers, rows: int = 8, i_chunk: int = 0, kernel: str = "warp_prefetch",
                 pad: bool = True):
        if not solvers:
            raise ValueError("BatchedSolver needs at least one solver")
        self.solvers = list(solvers)
        self._lib = _native.load()
        self._torch = self.solvers[0]._torch
        self.rows, self.i_chunk = rows, i_chunk
        if kernel not in PLAIN_KERNELS:
            raise ValueError(f"kernel must be one of {PLAIN_KERNELS}")
        self.kernel = kernel
        self.pad = pad  # members with nz % 4 != 0 run as padded twins (float4 tiles) in big runs
        h = ctypes.c_void_p()
        _native.check(self._lib.sf_batch_create(ctypes.byref(h)), "sf_batch_create")
        self._batch = h

    def __del__(self):
        b = getattr(self, "_batch", None)
        if b is not None and b.value:
            try:
                self._lib.sf_batch_destroy(b)
            except Exception:
                pass
            self._batch = None

    def _stream(self):
        return self._torch.cuda.current_stream().cuda_stream

    @staticmethod
    def steps_alone(s) -> bool:
        """Whether member ``s`` steps through its own plan within a run:
        plane boundaries or membrane sources (ordered passes after each step),
        or a nonuniform grid with ADE materials."""
        if any(hasattr(b, "plane_ops") for b in s._boundaries):
            return True
        if any(src.source_type == "membrane" for src in s._sources):
            return True
        return not s.grid.is_uniform and s.has_materials

    def _load(self, steps):
        """(Re)build the member list for a run of ``steps`` (int or per solver)."""
        torch = self._torch
        lib = self._lib
        _native.check(lib.sf_batch_clear(self._batch), "sf_batch_clear")
        _native.check(lib.sf_batch_set_tiles(self._batch, self.rows, self.i_chunk),
                      "sf_batch_set_tiles")
        _native.check(lib.sf_batch_set_kernel(self._batch, PLAIN_KERNELS.index(self.kernel)),
                      "sf_batch_set_kernel")
        counts = [int(steps)] * len(self.solvers) if np.isscalar(steps) else [int(n) for n in steps]
        if len(counts) != len(self.solvers):
            raise ValueError("one step count per solver")
        keep = []
        self._twins = []
        self._alone = []
        # padded twins give float4 items twice the size of scalar ones: they
        # pay when the run has work for every resident warp several times
        # over, and make small runs slower (fewer, larger items)
        busy = sum(int(np.prod(s.shape)) for s, n in zip(self.solvers, counts) if n)
        pad = self.pad and self.kernel != "column" and busy >= self.PAD_MIN_CELLS
        for s, n in zip(self.solvers, counts):
            if self.steps_alone(s):
                self._alone.append((s, n))
                continue
            vz_handed_out = s._host_exposed["vz"]  # the caller may have edited vz
            s._sync_tables()
            s._upload_exposed()
            src = s.source_table(n) if s._sources else None
            n_probe = len(s._probe_order)
            trace = (torch.empty((n, n_probe), dtype=torch.float32, device=s._device)
                     if n_probe and n else None)
            n_mic = getattr(s, "_mic_rows", 0)
            mics = (torch.empty((n, n_mic), dtype=torch.float32, device=s._device)
                    if n_mic and n else None)
            plan = s._plan
            twin = s._padded_twin(vz_handed_out) if pad and n else None
            if twin is not None:
                twin.copy_in(s)
                self._twins.append((s, twin))
                plan = twin.plan
            _native.check(lib.sf_batch_add_ex(self._batch, plan, n,
                                              None if src is None else src.data_ptr(),
                                              None if trace is None else trace.data_ptr(),
                                              None if mics is None else mics.data_ptr()),
                          "sf_batch_add")
            keep.append((s, n, src, trace, mics))
        return keep

    def autotune(self, launches: int = 3) -> dict:
        """Time the 9 tile shapes with each plain-tile kernel on the members'
        current state (unchanged) and keep the fastest.  Returns
        {(kernel, rows, i_chunk): ms per step, "best": (kernel, rows, i_chunk)}."""
        out = {}
        best = None
        for kernel in PLAIN_KERNELS:
            self.kernel = kernel
            self._load(1)
            ms = (ctypes.c_float * 9)()
            br, bc = ctypes.c_int(), ctypes.c_int()
            _native.check(self._lib.sf_batch_autotune(self._batch, int(launches), self._stream(),
                                                      ms, ctypes.byref(br), ctypes.byref(bc)),
                          "sf_batch_autotune")
            for a, r in enumerate((4, 8, 16)):
                for b, c in enumerate((8, 16, 32)):
                    t = float(ms[a * 3 + b])
                    out[(kernel, r, c)] = t
                    if t > 0 and (best is None or t < out[best]):
                        best = (kernel, r, c)
        self.kernel, self.rows, self.i_chunk = best
        out["best"] = best
        return out

    def run_steps(self, steps, graph_steps: int = 50) -> None:
        """Advance every member by ``steps`` (an int, or one count per
        solver) in one batched run; ``graph_steps`` > 0 replays CUDA graphs
        of that many steps."""
        import time as _time

        t0 = _time.perf_counter()
        keep = self._load(steps)
        t1 = _time.perf_counter()
        if keep:
            longest = max(n for _, n, _, _, _ in keep)
            _native.check(self._lib.sf_batch_run(self._batch, longest, int(graph_steps),
                                                 self._stream()), "sf_batch_run")
        self.host_s = {"load": t1 - t0, "run": _time.perf_counter() - t1}
        for s, twin in self._twins:
            twin.copy_out(s)
        for s, n, src, trace, mics in keep:
            if trace is not None:
                s._pending_traces.append((trace, list(s._probe_order)))
            times = []
            for _ in range(n):
                times.append(s._time)
                s._time += s.dt
            if mics is not None:
                s._pending_mics.append((mics, list(s._mic_order), times))
            if n:
                s._mark_device_newer()
                s._step_count += n
        for s, n in self._alone:  # their own plans, queued after the batch on the same stream
            if n:
                s.run_steps(n)
        self._keepalive = keep  # tables stay alive until the stream has used them

    @property
    def cell_updates(self):
        return sum(int(np.prod(s.shape)) for s in self.solvers)
