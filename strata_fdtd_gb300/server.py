"""A served stream of independent solves with continuous batching.

Requests (each a fully configured FDTD solve and a step count) arrive over
time.  The server keeps every admitted solve's fields, flags, PML tables and
ADE state resident in HBM and advances all of them together in step groups
(one batched persistent launch per time step, see batch.py).  At every group
boundary it retires finished solves (freeing their memory) and admits the
requests that have arrived, first come first served, as long as the sum of
their exact device footprints stays within the HBM budget.  A solve's result
is bit-identical whether it ran alone or in the mix.

The scheduling logic is independent of the GPU: it drives an *executor*
(``GPUExecutor`` here; tests substitute a fake one to exercise admission,
failures and cancellation on the CPU).

Failure handling (no GPU fault is involved in any of it): a request whose
footprint exceeds the whole budget is rejected at submission; a request whose
construction raises (malformed spec, failed allocation) is marked failed and
the server carries on; a request can be cancelled before or while it runs;
a solve whose pressure turns non-finite is stopped and marked failed.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Any, Callable

import numpy as np


@dataclass
class Request:
    """One solve: ``build()`` returns a configured solver (it is called only
    when the request is admitted), ``steps`` time steps, ``arrival`` seconds
    after the stream starts, ``nbytes`` its device footprint."""

    rid: int
    build: Callable[[], Any]
    steps: int
    arrival: float = 0.0
    nbytes: int = 0
    status: str = "queued"
    error: str | None = None
    t_admit: float | None = None
    t_done: float | None = None
    result: dict | None = None
    remaining: int = 0
    handle: Any = None
    cancel_requested: bool = False
    cell_updates: int = 0
    cells: int = 0
    last_group: int = -1      # index of the group that enqueued its last steps
    collect: Any = None       # pipelined executors: waits for and returns the result

    done_event: Any = None    # set when the request leaves the server (posted requests)

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.arrival

    def wait(self, timeout: float | None = None) -> bool:
        """For a request given to a running server (``SolveServer.post``):
        block until it is done, failed, rejected or cancelled; False on
        timeout."""
        if self.done_event is None:
            raise RuntimeError("wait() is for requests posted to a running server")
        return self.done_event.wait(timeout)


def solve_bytes(shape, geometry=True, debye_poles=0, lorentz_poles=0, probes=2, sources=1) -> int:
    """Exact device bytes one solve holds: two ping-pong sets of p, vx, vy,
    vz (32 B/cell), the geometry mask and the flag byte (2 B/cell with a
    geometry), material ids (1 B/cell with ADE), 4 B/cell per Debye and
    8 B/cell per Lorentz auxiliary field, plus PML decays, probe cells and
    the energy scratch."""
    nx, ny, nz = shape
    n = nx * ny * nz
    b = 32 * n + (2 * n if geometry else 0)
    if debye_poles or lorentz_poles:
        b += n + 4 * n * debye_poles + 8 * n * lorentz_poles
    b += 4 * (nx + ny + nz) + 8 * probes + 8 * sources
    return b


class SolveServer:
    """Continuous-batching request loop over ``executor``.

    ``hbm_budget``: bytes of device memory the resident solves may hold;
    ``step_group``: time steps between admission points;
    ``max_active``: cap on concurrently resident solves;
    ``max_active_cells``: cap on the cells of the running solves (None: no
    cap).  Enough cells to fill the device keep the throughput while fewer
    solves share it, so each finishes sooner (first come, first served
    instead of processor sharing); a solve larger than the cap still runs,
    alone."""

    def __init__(self, executor, hbm_budget: float = 160e9, step_group: int = 250,
                 max_active: int = 512, max_active_cells: int | None = None,
                 clock=time.perf_counter):
        self.ex = executor
        self.budget = int(hbm_budget)
        self.step_group = int(step_group)
        self.max_active = int(max_active)
        self.max_cells = None if max_active_cells is None else int(max_active_cells)
        self.active_cells = 0
        self.clock = clock
        self.queue: list[Request] = []
        self.active: list[Request] = []
        self.finished: list[Request] = []
        self.in_use = 0
        self.peak_in_use = 0
        self.peak_active = 0
        self.groups = 0

    def _finish(self, r: Request) -> None:
        self.finished.append(r)
        if r.done_event is not None:
            r.done_event.set()

    # -- submission ----------------------------------------------------------
    def submit(self, req: Request) -> Request:
        if req.nbytes > self.budget:
            req.status, req.error = "rejected", (
                f"needs {req.nbytes} bytes, above the {self.budget}-byte budget")
            self._finish(req)
            return req
        req.remaining = int(req.steps)
        self.queue.append(req)
        return req

    def cancel(self, rid: int) -> bool:
        for r in self.queue + self.active:
            if r.rid == rid:
                r.cancel_requested = True
                return True
        return False

    # -- serving in the background ---------------------------------------------
    def start(self) -> "SolveServer":
        """Serve in a background thread: requests given to ``post`` from any
        thread join at the next group boundary, as arrivals at the time they
        are posted.  ``stop`` ends the thread."""
        if getattr(self, "_thread", None) is not None:
            raise RuntimeError("the server is already running")
        self._inbox: queue.SimpleQueue = queue.SimpleQueue()
        self._stop_req = threading.Event()
        self._drain_on_stop = True
        self.t0 = self.clock()
        self._thread = threading.Thread(target=self._serve, name="solve-server", daemon=True)
        self._thread.start()
        return self

    def post(self, req: Request) -> Request:
        """Hand a request to the running server (thread-safe); its
        ``wait()`` returns once it has left the server."""
        if getattr(self, "_thread", None) is None:
            raise RuntimeError("post() needs a started server (start())")
        if not self._thread.is_alive():
            raise RuntimeError("the serving thread has stopped") from getattr(self, "error", None)
        req.done_event = threading.Event()
        req.arrival = self.clock() - self.t0
        self._inbox.put(req)
        return req

    def stop(self, drain: bool = True, timeout: float | None = None) -> dict:
        """Stop the background thread: with ``drain`` after every posted
        request has finished, else cancelling the queued and running ones.
        Returns the statistics."""
        if getattr(self, "_thread", None) is None:
            raise RuntimeError("stop() needs a started server (start())")
        self._drain_on_stop = drain
        self._stop_req.set()
        self._thread.join(timeout)
        self._thread = None
        if getattr(self, "error", None) is not None:
            raise RuntimeError("the serving thread stopped on an error") from self.error
        return self.stats()

    def _drain_inbox(self) -> None:
        inbox = getattr(self, "_inbox", None)
        while inbox is not None:
            try:
                req = inbox.get_nowait()
            except queue.Empty:
                return
            self.submit(req)

    def _serve(self) -> None:
        """The background loop; an error in it fails every request still
        held (so no ``wait`` blocks for ever) and is re-raised by ``stop``."""
        self.error = None
        try:
            self._serve_loop()
        except BaseException as e:  # noqa: BLE001 - reported through stop()
            self.error = e
            t = self.clock() - self.t0
            self._drain_inbox()
            for r in self.queue + self.active:
                r.status, r.error, r.t_done = "failed", f"server error: {e!r}", t
                self._finish(r)
            self.queue, self.active = [], []

    def _serve_loop(self) -> None:
        def now():
            return self.clock() - self.t0

        while True:
            self._drain_inbox()
            if self._stop_req.is_set():
                if not self._drain_on_stop:
                    for r in self.queue + self.active:
                        r.cancel_requested = True
                if not (self.queue or self.active):
                    return
            if self.queue or self.active:
                if getattr(self.ex, "pipelined", False):
                    self._run_pipelined(now, True)
                else:
                    self._run_simple(now, True)
                continue
            try:  # idle: wait for the next request
                self.submit(self._inbox.get(timeout=0.02))
            except queue.Empty:
                pass

    # -- scheduling ----------------------------------------------------------
    def _admit(self, now: float) -> None:
        self._drain_inbox()
        stop = getattr(self, "_stop_req", None)
        if stop is not None and stop.is_set() and not self._drain_on_stop:
            for r in self.queue + self.active:  # stop(drain=False): cancel the rest
                r.cancel_requested = True
        keep = []
        for r in self.queue:
            if r.cancel_requested:
                r.status, r.t_done = "cancelled", now
                self._finish(r)
                continue
            fits_cells = (self.max_cells is None or not self.active
                          or self.active_cells + r.cells <= self.max_cells)
            if (r.arrival <= now and len(self.active) < self.max_active
                    and self.in_use + r.nbytes <= self.budget and fits_cells
                    and not keep):  # first come, first served: no overtaking
                try:
                    r.handle = self.ex.start(r)
                except Exception as e:  # malformed request or failed allocation
                    r.status, r.error, r.t_done = "failed", f"{type(e).__name__}: {e}", now
                    self._finish(r)
                    continue
                r.status, r.t_admit = "running", now
                self.in_use += r.nbytes
                self.active_cells += r.cells
                self.active.append(r)
            else:
                keep.append(r)
        self.queue = keep
        self.peak_in_use = max(self.peak_in_use, self.in_use)
        self.peak_active = max(self.peak_active, len(self.active))

    def _retire(self, now: float) -> None:
        still = []
        for r in self.active:
            done = r.remaining <= 0
            bad = self.ex.failed(r.handle)
            if done or bad or r.cancel_requested:
                if bad:
                    r.status, r.error = "failed", bad
                elif r.cancel_requested and not done:
                    r.status = "cancelled"
                else:
                    r.status = "done"
                    r.result = self.ex.finish(r.handle)
                self.ex.release(r.handle)
                r.handle = None
                r.t_done = now
                self.in_use -= r.nbytes
                self.active_cells -= r.cells
                self._finish(r)
            else:
                still.append(r)
        self.active = still

    def run(self, requests=(), realtime: bool = True) -> dict:
        """Serve ``requests`` (plus anything submitted before) to completion.
        With ``realtime`` the arrival times are honoured against the clock;
        otherwise every request counts as arrived at the start."""
        for r in requests:
            self.submit(r)
        t0 = self.clock()
        self.t0 = t0

        def now():
            return self.clock() - t0

        if getattr(self.ex, "pipelined", False):
            return self._run_pipelined(now, realtime)
        return self._run_simple(now, realtime)

    def _run_simple(self, now, realtime: bool) -> dict:
        """One group at a time: admit, advance, wait, retire."""
        while self.queue or self.active:
            self._admit(now() if realtime else float("inf"))
            if not self.active:
                if not self.queue:
                    break
                wait = min(r.arrival for r in self.queue) - now()
                if realtime and wait > 0:
                    time.sleep(min(wait, 0.01))
                continue
            members = list(self.active)
            counts = [min(self.step_group, r.remaining) for r in members]
            self.ex.advance([r.handle for r in members], counts)
            # requests that arrived meanwhile are set up while the GPU works;
            # they join from the next group
            if realtime:
                self._admit(now())
            self.ex.wait()
            for r, n in zip(members, counts):
                r.remaining -= n
                r.cell_updates += n * self.ex.cells(r.handle)
            self.groups += 1
            self._retire(now())
        return self.stats()

    def _run_pipelined(self, now, realtime: bool) -> dict:
        """The same loop with one group in flight: group g+1 is built and
        queued while the device runs group g, and group g's solves are
        retired once it has completed (its finished solves' results were
        queued for copy-out right behind it).  Solves whose steps are all
        queued stop counting against the cell cap at once and free their
        memory budget when they retire; a non-finite pressure is caught one
        group later."""
        pending = None  # (token, members, group index) of the group in flight
        self._release_later = []
        while self.queue or self.active or pending is not None:
            self._admit(now() if realtime else float("inf"))
            group = None
            if self.active:
                members = list(self.active)
                counts = [min(self.step_group, r.remaining) for r in members]
                self.ex.advance([r.handle for r in members], counts)
                gi = self.groups
                self.groups += 1
                still = []
                for r, n in zip(members, counts):
                    r.remaining -= n
                    r.cell_updates += n * self.ex.cells(r.handle)
                    r.last_group = gi
                    if r.remaining > 0 and not r.cancel_requested:
                        still.append(r)
                        continue
                    self.active_cells -= r.cells
                    if r.remaining <= 0:  # its result follows the group on the stream
                        r.collect = self.ex.collect(r.handle)
                self.active = still
                group = (self.ex.mark(), members, gi)
                if realtime:  # arrivals are set up while the device works
                    self._admit(now())
            elif pending is None:
                if not self.queue:
                    break
                wait = min(r.arrival for r in self.queue) - now()
                if realtime and wait > 0:
                    time.sleep(min(wait, 0.01))
                continue
            if pending is not None:
                self.ex.wait_for(pending[0])
                done_gi = pending[2]
                keep = []
                for last, h in self._release_later:
                    if last <= done_gi:
                        self.ex.release(h)
                    else:
                        keep.append((last, h))
                self._release_later = keep
                self._retire_group(pending[1], pending[2], now())
            pending = group
        return self.stats()

    def _retire_group(self, members, gi: int, now: float) -> None:
        """Retire the members of completed group gi that are finished (their
        last steps were in it), failed or cancelled."""
        for r in members:
            if r.status != "running":
                continue
            bad = self.ex.failed(r.handle)
            if not bad and not r.cancel_requested and not (r.remaining <= 0 and r.last_group == gi):
                continue
            if bad:
                r.status, r.error = "failed", bad
            elif r.cancel_requested and r.remaining > 0:
                r.status = "cancelled"
            else:
                r.status = "done"
                r.result = r.collect() if r.collect is not None else self.ex.finish(r.handle)
            if r in self.active:  # stopped early (failed or cancelled while still stepping)
                self.active.remove(r)
                self.active_cells -= r.cells
            r.collect = None
            if r.last_group > gi:  # a group still in flight uses it: release after that
                self._release_later.append((r.last_group, r.handle))
            else:
                self.ex.release(r.handle)
            r.handle = None
            r.t_done = now
            self.in_use -= r.nbytes
            self._finish(r)

    def stats(self) -> dict:
        done = [r for r in self.finished if r.status == "done"]
        lat = np.array([r.latency for r in done]) if done else np.zeros(0)
        span = max((r.t_done for r in done), default=0.0)
        cu = sum(r.cell_updates for r in done)
        return {
            "requests": len(self.finished), "done": len(done),
            "failed": sum(r.status == "failed" for r in self.finished),
            "rejected": sum(r.status == "rejected" for r in self.finished),
            "cancelled": sum(r.status == "cancelled" for r in self.finished),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "mean_latency_s": float(lat.mean()) if lat.size else None,
            "makespan_s": span, "cell_updates": cu,
            "gcell_updates_per_s": cu / span / 1e9 if span > 0 else None,
            "peak_hbm_bytes": self.peak_in_use, "peak_active": self.peak_active,
            "step_groups": self.groups,
            "errors": [(r.rid, r.status, r.error) for r in self.finished
                       if r.status in ("failed", "rejected")][:20],
        }


class GPUExecutor:
    """Runs the admitted solves on the GPU: construction on a side stream
    (overlapping the running group), each group as one batched run.  Solves
    of ``solo_cells`` cells or more fill the device by themselves and step
    through the single-grid column kernels instead (same results, a faster
    kernel for one large grid); None batches everything."""

    def __init__(self, graph_steps: int = 50, solo_cells: int | None = 1 << 24,
                 batch_min_cells: int = 0):
        import torch

        from .batch import BatchedSolver

        self.torch = torch
        self.Batched = BatchedSolver
        self.graph_steps = graph_steps
        self.solo_cells = solo_cells
        # a group whose batchable solves hold fewer cells than this steps them
        # one by one through the single-grid path instead (the tail of a
        # stream, when a few small solves are left)
        self.batch_min_cells = int(batch_min_cells)
        self.host_advance_s = 0.0  # host time spent enqueueing groups
        self.host_wait_s = 0.0     # host time blocked on the device
        # groups run on a stream of their own: the library's synchronous
        # set-up copies (legacy default stream) then never wait for them
        self.side = torch.cuda.Stream()
        self.main = torch.cuda.Stream()
        self._pending = None
        self._new: list = []
        self._groups: list = []  # groups queued and not yet waited for
        self.host_s: dict = {}   # host time by part of a group's set-up

    host_build_s = 0.0  # host time constructing admitted solves

    def start(self, req):
        t0 = time.perf_counter()
        with self.torch.cuda.stream(self.side):
            s = req.build()
            # the rest of the set-up a run would do first (device tables, ADE
            # fields, the padded twin for odd nz) happens here, on the side
            # stream: its blocking host-to-device copies then wait for this
            # stream only, not for the group running on the main one
            s._sync_tables()
            s._upload_exposed()
            if self.solo_cells is None or int(np.prod(s.shape)) < self.solo_cells:
                s._padded_twin(False)
        self.host_build_s += time.perf_counter() - t0
        self._new.append(s)
        return {"solver": s, "bad": None}

    def advance(self, handles, counts):
        with self.torch.cuda.stream(self.main):
            self._advance(handles, counts)

    def _advance(self, handles, counts):
        t0 = time.perf_counter()
        if self._new:
            self.main.wait_stream(self.side)
            self._new = []
        batch, steps = [], []
        for h, n in zip(handles, counts):
            s = h["solver"]
            if self.solo_cells is not None and int(np.prod(s.shape)) >= self.solo_cells:
                s.run_steps(n)
            else:
                batch.append(s)
                steps.append(n)
        self._tick("solo", t0)
        t1 = time.perf_counter()
        b = None
        if batch and sum(int(np.prod(s.shape)) for s in batch) < self.batch_min_cells:
            for s, n in zip(batch, steps):
                s.run_steps(n)
            batch = []
        if batch:
            b = self.Batched(batch)
            b.run_steps(steps, graph_steps=self.graph_steps)
            for k, v in b.host_s.items():
                self.host_s["batch_" + k] = self.host_s.get("batch_" + k, 0.0) + v
        self._tick("batch", t1)
        self._pending = (b, handles)
        t2 = time.perf_counter()
        self._queue_checks(handles)
        self._tick("checks", t2)
        self.host_advance_s += time.perf_counter() - t0

    def _tick(self, part, t0):
        self.host_s[part] = self.host_s.get(part, 0.0) + time.perf_counter() - t0

    # -- one group in flight (SolveServer's pipelined loop) ------------------
    pipelined = True

    def _queue_checks(self, handles):
        """Copy the last probe row of each solve's new trace to pinned host
        memory behind the group, for the non-finite check."""
        torch = self.torch
        checks = []
        for h in handles:
            s = h["solver"]
            if s is not None and s._pending_traces:
                tr = s._pending_traces[-1][0]
                row = torch.empty((1, tr.shape[1]), dtype=tr.dtype, pin_memory=True)
                row.copy_(tr[-1:], non_blocking=True)
                checks.append((h, row))
        self._groups.append({"batch": self._pending[0], "checks": checks, "event": None})

    def mark(self):
        """A token for the group just queued: a CUDA event behind it."""
        ev = self.torch.cuda.Event()
        ev.record(self.main)
        rec = self._groups[-1]
        rec["event"] = ev
        self._pending = None
        return rec

    def collect(self, h):
        """Queue the copy-out of a finished solve's traces; returns the
        function that waits for it and gives the result."""
        t0 = time.perf_counter()
        with self.torch.cuda.stream(self.main):
            out = h["solver"].probe_data_async()
        self._tick("collect", t0)
        return out

    def wait_for(self, rec):
        t0 = time.perf_counter()
        rec["event"].synchronize()
        self.host_wait_s += time.perf_counter() - t0
        for h, row in rec["checks"]:
            if not np.all(np.isfinite(row.numpy())):
                h["bad"] = "pressure became non-finite at a probe"
        self._groups.remove(rec)

    def wait(self):
        t0 = time.perf_counter()
        self.main.synchronize()
        self.host_wait_s += time.perf_counter() - t0
        if self._pending is not None:
            _, handles = self._pending
            for h in handles:
                traces = h["solver"].get_probe_data()
                if any(len(t) and not np.all(np.isfinite(t[-1:])) for t in traces.values()):
                    h["bad"] = "pressure became non-finite at a probe"
            self._pending = None

    def failed(self, h):
        return h["bad"]

    def cells(self, h):
        return int(np.prod(h["solver"].shape))

    def finish(self, h):
        return h["solver"].get_probe_data()

    def release(self, h):
        h["solver"] = None


class SequentialExecutor(GPUExecutor):
    """The baseline: one solve at a time through the single-grid path."""

    def _advance(self, handles, counts):
        t0 = time.perf_counter()
        if self._new:
            self.main.wait_stream(self.side)
            self._new = []
        for h, n in zip(handles, counts):
            h["solver"].run_steps(n)
        self._pending = (None, handles)
        self._queue_checks(handles)
        self.host_advance_s += time.perf_counter() - t0
