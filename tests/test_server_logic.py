"""The serving loop's scheduling on the CPU, with a fake executor: FIFO
admission against the HBM budget, continuous batching (arrivals join at
group boundaries while others run), rejection of oversized requests, failed
construction, cancellation and non-finite detection.  No GPU involved."""
import numpy as np

from strata_fdtd_gb300.server import Request, SolveServer, solve_bytes


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    """Each advanced step costs 1 ms of fake time; records group membership."""

    def __init__(self, clock, fail_build=(), nan_after=None):
        self.clock = clock
        self.groups = []
        self.fail_build = set(fail_build)
        self.nan_after = nan_after or {}
        self.done_steps = {}

    def start(self, req):
        if req.rid in self.fail_build:
            raise MemoryError("simulated allocation failure")
        self.done_steps[req.rid] = 0
        return {"rid": req.rid, "bad": None}

    def advance(self, handles, counts):
        self.groups.append(sorted(h["rid"] for h in handles))
        for h, n in zip(handles, counts):
            self.done_steps[h["rid"]] += n
            lim = self.nan_after.get(h["rid"])
            if lim is not None and self.done_steps[h["rid"]] >= lim:
                h["bad"] = "pressure became non-finite at a probe"
        self.clock.t += 1e-3 * max(counts)

    def wait(self):
        pass

    def failed(self, h):
        return h["bad"]

    def cells(self, h):
        return 1000

    def finish(self, h):
        return {"steps": self.done_steps[h["rid"]]}

    def release(self, h):
        pass


def _req(rid, steps, arrival=0.0, nbytes=10):
    return Request(rid=rid, build=lambda: None, steps=steps, arrival=arrival, nbytes=nbytes)


def test_budget_limits_residency_and_fifo_order():
    clock = FakeClock()
    ex = FakeExecutor(clock)
    srv = SolveServer(ex, hbm_budget=30, step_group=10, clock=clock)
    reqs = [_req(q, 25, nbytes=10) for q in range(6)]
    stats = srv.run(reqs, realtime=False)
    assert stats["done"] == 6 and stats["peak_hbm_bytes"] <= 30
    assert max(len(g) for g in ex.groups) == 3
    assert ex.groups[0] == [0, 1, 2]
    # FIFO: request 3 only runs after one of the first three finished
    first_with_3 = next(i for i, g in enumerate(ex.groups) if 3 in g)
    assert all(len(g) == 3 for g in ex.groups[:first_with_3])
    assert all(r.result["steps"] == 25 for r in srv.finished)


def test_continuous_batching_admits_arrivals_between_groups():
    clock = FakeClock()
    ex = FakeExecutor(clock)
    srv = SolveServer(ex, hbm_budget=1000, step_group=10, clock=clock)
    reqs = [_req(0, 100, arrival=0.0), _req(1, 30, arrival=0.025), _req(2, 10, arrival=0.05)]
    srv.run(reqs, realtime=True)
    joined = {rid: next(i for i, g in enumerate(ex.groups) if rid in g) for rid in (0, 1, 2)}
    assert joined[0] == 0 and 0 < joined[1] < joined[2]
    # request 1 overlapped with request 0 (same groups), not queued behind it
    assert any(set(g) >= {0, 1} for g in ex.groups)
    done = {r.rid: r for r in srv.finished}
    assert all(done[q].status == "done" for q in (0, 1, 2))
    assert done[2].latency < done[0].latency


def test_rejection_failure_cancel_and_nonfinite():
    clock = FakeClock()
    ex = FakeExecutor(clock, fail_build={2}, nan_after={3: 20})
    srv = SolveServer(ex, hbm_budget=100, step_group=10, clock=clock)
    reqs = [_req(0, 40), _req(1, 40, nbytes=500), _req(2, 40), _req(3, 60), _req(4, 80)]
    for r in reqs:
        srv.submit(r)
    srv.cancel(4)
    stats = srv.run(realtime=False)
    st = {r.rid: r.status for r in srv.finished}
    assert st == {0: "done", 1: "rejected", 2: "failed", 3: "failed", 4: "cancelled"}
    errs = {r.rid: r.error for r in srv.finished}
    assert "budget" in errs[1] and "MemoryError" in errs[2] and "non-finite" in errs[3]
    assert stats["done"] == 1 and stats["failed"] == 2


def test_solve_bytes_counts_every_buffer():
    n = 40 * 50 * 60
    assert solve_bytes((40, 50, 60), geometry=False, probes=0, sources=0) == 32 * n + 4 * 150
    assert solve_bytes((40, 50, 60), geometry=True, debye_poles=2, probes=2, sources=1) == (
        32 * n + 2 * n + n + 8 * n + 4 * 150 + 16 + 8)
    assert np.isclose(solve_bytes((320, 320, 320)) / 1e9, 1.11, atol=0.02)


def test_cell_cap_admits_in_order_and_lets_an_oversized_solve_run_alone():
    clock = FakeClock()
    ex = FakeExecutor(clock)
    srv = SolveServer(ex, hbm_budget=10**9, step_group=10, max_active_cells=300, clock=clock)
    reqs = [Request(rid=q, build=lambda: None, steps=20, nbytes=1, cells=c)
            for q, c in enumerate([100, 100, 100, 500, 100, 200])]
    stats = srv.run(reqs, realtime=False)
    assert stats["done"] == 6
    assert ex.groups[0] == [0, 1, 2]          # 300 cells: at the cap
    assert [3] in ex.groups                   # 500 cells > cap: runs, alone
    assert not any(3 in g and len(g) > 1 for g in ex.groups)
    assert ex.groups[-1] == [4, 5]            # admitted together after it
    assert srv.active_cells == 0


class FakePipelinedExecutor(FakeExecutor):
    """The pipelined interface: groups are queued (advance + mark), their
    effects become visible only when waited for (wait_for), and a finished
    solve's result is collected from a copy queued behind its last group."""

    pipelined = True

    def __init__(self, clock, **kw):
        super().__init__(clock, **kw)
        self.queued = []      # group records not yet waited for
        self.completed = set()
        self.max_in_flight = 0

    def advance(self, handles, counts):
        super().advance(handles, counts)
        self.queued.append(len(self.groups) - 1)
        self.max_in_flight = max(self.max_in_flight, len(self.queued))

    def mark(self):
        return self.queued[-1]

    def wait_for(self, token):
        assert token == self.queued[0], "groups complete in queue order"
        self.queued.pop(0)
        self.completed.add(token)

    def collect(self, h):
        rid, steps, group = h["rid"], self.done_steps[h["rid"]], len(self.groups) - 1

        def result():
            assert group in self.completed, "result read before its group completed"
            return {"steps": steps}

        return result


def test_pipelined_loop_keeps_one_group_in_flight_and_retires_after_completion():
    clock = FakeClock()
    ex = FakePipelinedExecutor(clock, nan_after={4: 30})
    srv = SolveServer(ex, hbm_budget=30, step_group=10, clock=clock)
    for q in range(6):
        srv.submit(_req(q, 25 + 5 * q, nbytes=10))
    assert srv.cancel(5)
    stats = srv.run(realtime=False)
    assert ex.max_in_flight == 2 and not ex.queued
    assert stats["peak_hbm_bytes"] <= 30
    by = {r.rid: r for r in srv.finished}
    for q in (0, 1, 2, 3):
        assert by[q].status == "done" and by[q].result == {"steps": 25 + 5 * q}, by[q]
    assert by[4].status == "failed" and "non-finite" in by[4].error
    assert by[5].status == "cancelled"
    assert srv.in_use == 0 and srv.active_cells == 0 and not srv.active
    # FIFO admission: request 3 joins only after one of the first three left
    first_with_3 = next(i for i, g in enumerate(ex.groups) if 3 in g)
    assert all(3 not in g for g in ex.groups[:first_with_3])
    assert all(len(g) <= 3 for g in ex.groups)


def test_background_server_takes_posts_from_threads():
    """start() / post() / wait() / stop(): requests posted from several
    threads while the server runs are admitted at group boundaries and each
    wait() returns once its request is done; an oversized one is rejected at
    once; stop(drain=False) cancels what is still queued or running."""
    import threading
    import time as _time

    class SlowExecutor(FakeExecutor):
        def advance(self, handles, counts):
            super().advance(handles, counts)
            _time.sleep(0.001)

    ex = SlowExecutor(FakeClock())
    srv = SolveServer(ex, hbm_budget=100, step_group=10, clock=_time.perf_counter).start()
    posted = []
    lock = threading.Lock()

    def client(base):
        for q in range(5):
            r = srv.post(_req(base + q, steps=25 + 5 * q, nbytes=10))
            with lock:
                posted.append(r)
            _time.sleep(0.002)

    threads = [threading.Thread(target=client, args=(100 * k,)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    big = srv.post(_req(999, steps=10, nbytes=1000))
    assert big.wait(5) and big.status == "rejected"
    for r in posted:
        assert r.wait(10), r.rid
        assert r.status == "done" and r.result == {"steps": r.steps}
        assert r.latency is not None and r.latency >= 0
    late = [srv.post(_req(500 + q, steps=10**6, nbytes=10)) for q in range(3)]
    st = srv.stop(drain=False, timeout=10)
    assert all(r.status == "cancelled" for r in late)
    assert st["done"] == 15 and st["rejected"] == 1 and st["cancelled"] == 3
    assert max(len(g) for g in ex.groups) > 1  # posts shared groups


def test_background_server_error_fails_held_requests():
    """An executor error inside the serving thread fails every request the
    server still holds (their wait() returns) and stop() raises it."""
    import time as _time

    import pytest

    class Broken(FakeExecutor):
        def advance(self, handles, counts):
            raise RuntimeError("device lost")

    srv = SolveServer(Broken(FakeClock()), hbm_budget=100, step_group=10,
                      clock=_time.perf_counter).start()
    reqs = [srv.post(_req(q, steps=50)) for q in range(3)]
    for r in reqs:
        assert r.wait(5)
        assert r.status == "failed" and "device lost" in r.error
    with pytest.raises(RuntimeError):
        srv.stop(timeout=5)
    with pytest.raises(RuntimeError):
        SolveServer(FakeExecutor(FakeClock())).stop()
