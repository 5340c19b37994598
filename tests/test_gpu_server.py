"""The served stream on the GPU: requests arriving while others run are
admitted between step groups and overlap on the device; every result must
be bit-identical to the same request solved alone (tolerance: none)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from strata_fdtd_gb300.server import GPUExecutor, SolveServer  # noqa: E402
from strata_fdtd_gb300.workloads import served_stream  # noqa: E402


def test_served_results_equal_alone_and_requests_overlap():
    reqs = served_stream(seed=7, n_requests=10, rate=400.0, edges=(40, 72), steps=(60, 240),
                         pml=(4, 8), ade_fraction=0.5)
    alone = served_stream(seed=7, n_requests=10, rate=400.0, edges=(40, 72), steps=(60, 240),
                          pml=(4, 8), ade_fraction=0.5)
    srv = SolveServer(GPUExecutor(graph_steps=0), hbm_budget=160e9, step_group=40)
    stats = srv.run(reqs, realtime=True)
    assert stats["done"] == 10, stats["errors"]
    assert stats["peak_active"] > 1
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0
    results = {r.rid: r.result for r in srv.finished}
    for r in alone:
        s = r.build()
        s.run_steps(r.steps)
        ref = s.get_probe_data()
        for name, tr in ref.items():
            np.testing.assert_array_equal(results[r.rid][name], tr, err_msg=f"request {r.rid}")
        assert len(ref["near"]) == r.steps


def test_budget_holds_on_the_gpu():
    reqs = served_stream(seed=11, n_requests=6, rate=1e6, edges=(40, 56), steps=(30, 60),
                         pml=(4, 6), ade_fraction=0.0)
    budget = 2.5 * max(r.nbytes for r in reqs)
    srv = SolveServer(GPUExecutor(), hbm_budget=budget, step_group=20)
    stats = srv.run(reqs, realtime=False)
    assert stats["done"] == 6, stats
    assert stats["peak_hbm_bytes"] <= budget
    # smaller solves may fit three at a time, never all six
    assert 1 <= stats["peak_active"] < 6
