"""Batched solves: many FDTDSolver instances stepped together on one GPU.

Each member is an ordinary, fully configured :class:`FDTDSolver` (grid size,
geometry, PML, sources, probes and ADE materials may all differ).  A run
issues, per time step, one persistent launch whose blocks pull
(grid, i-chunk, rows, columns) tiles from a device work queue
(``sf_batch_*`` in include/sf_gb300.h); members with fewer steps drop out
when they are done.  Every member's fields, traces and auxiliary ADE fields
are bit-identical to running it alone.  No counterpart in the reference,
which steps one solver at a time.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


PLAIN_KERNELS = ("column", "warp", "warp_prefetch", "warp_prefetch_m8")


class BatchedSolver:
    """Steps ``solvers`` together.  ``rows`` (4, 8, 16) and ``i_chunk``
    (planes per tile, 0 = 16) set the tile shape and ``kernel`` (one of
    PLAIN_KERNELS) the kernel of the tiles away from material boxes;
    :meth:`autotune` picks all three."""

    def __init__(self, solvers, rows: int = 8, i_chunk: int = 0, kernel: str = "warp_prefetch"):
        if not solvers:
            raise ValueError("BatchedSolver needs at least one solver")
        if any(s._microphones for s in solvers):
            raise NotImplementedError("microphones are recorded by single-solver runs only")
        if any(getattr(s, "_plane_bc_dirty", False) or
               any(hasattr(b, "plane_ops") for b in s._boundaries) for s in solvers):
            raise NotImplementedError("plane boundaries are stepped by single-solver runs only")
        if any(src.source_type == "membrane" for s in solvers for src in s._sources):
            raise NotImplementedError("membrane sources are stepped by single-solver runs only")
        if any(not s.grid.is_uniform for s in solvers):
            raise NotImplementedError("nonuniform grids are stepped by single-solver runs only")
        self.solvers = list(solvers)
        self._lib = _native.load()
        self._torch = self.solvers[0]._torch
        self.rows, self.i_chunk = rows, i_chunk
        if kernel not in PLAIN_KERNELS:
            raise ValueError(f"kernel must be one of {PLAIN_KERNELS}")
        self.kernel = kernel
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
        for s, n in zip(self.solvers, counts):
            s._sync_tables()
            s._upload_exposed()
            src = s.source_table(n) if s._sources else None
            n_probe = len(s._probe_order)
            trace = (torch.empty((n, n_probe), dtype=torch.float32, device=s._device)
                     if n_probe and n else None)
            _native.check(lib.sf_batch_add(self._batch, s._plan, n,
                                           None if src is None else src.data_ptr(),
                                           None if trace is None else trace.data_ptr()),
                          "sf_batch_add")
            keep.append((s, n, src, trace))
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
        keep = self._load(steps)
        longest = max(n for _, n, _, _ in keep)
        _native.check(self._lib.sf_batch_run(self._batch, longest, int(graph_steps),
                                             self._stream()), "sf_batch_run")
        for s, n, src, trace in keep:
            if trace is not None:
                s._pending_traces.append((trace, list(s._probe_order)))
            if n:
                s._mark_device_newer()
                s._step_count += n
                for _ in range(n):
                    s._time += s.dt
        self._keepalive = keep  # tables stay alive until the stream has used them

    @property
    def cell_updates(self):
        return sum(int(np.prod(s.shape)) for s in self.solvers)
