"""The multi-GPU form is replicas only: each rank steps its own copy of the
workload with no collective on the data path; the bench line reports the
whole-job rate over the slowest rank's time.  This checks that host logic
with two gloo ranks on the CPU (no GPU involved)."""
import os
import socket
import sys
import types

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slow = bench.max_over_ranks(1.5 + rank, dist, "cpu")  # rank 1 is slower
        rate = bench.replica_rate(world, 64_000_000 * 100 * 40, slow)
        out[rank] = (slow, rate)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job_rate():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, join=True,
                           start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]                  # every rank prints the same numbers
    slow, rate = res[0]
    assert slow == 2.5                       # max over ranks, not rank 0's own time
    assert rate == pytest.approx(2 * 64e6 * 100 * 40 / 2.5 / 1e9)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.replica_rate(1, 10**9, 1.0) == 1.0


def test_bench_extras_report_a_failing_part_and_keep_the_rest(monkeypatch):
    """A sub-benchmark that raises becomes {"error": ...} in its key; the
    other parts, and so the printed line, are still produced."""
    import bench

    def boom(args):
        raise RuntimeError("no device")

    monkeypatch.setattr(bench, "run_batch", boom)
    monkeypatch.setattr(bench, "run_serve", lambda args: {
        "value": 1.0, "unit": "u", "config": {"workload": "w"}, "throughput_ratio": 1.0,
        "results_identical": True,
        "served": {"p50_latency_s": 1.0, "p99_latency_s": 2.0, "makespan_s": 3.0, "done": 4,
                   "peak_active": 5},
        "sequential": {"gcell_updates_per_s": 0.5, "p50_latency_s": 1.5, "p99_latency_s": 2.5}})
    monkeypatch.setattr(bench, "run_adjoint", boom)
    monkeypatch.setattr(bench, "parity_quick_start", lambda: {"ok": True})
    args = types.SimpleNamespace(max_active_cells=1 << 28)
    out = bench.extras(args)
    assert out["batched"] == {"error": "RuntimeError: no device"}
    assert out["adjoint"] == {"error": "RuntimeError: no device"}
    assert out["served"]["value"] == 1.0 and out["served"]["max_active_cells"] == 1 << 28
    assert out["parity"]["quick_start_100"] == {"ok": True}
