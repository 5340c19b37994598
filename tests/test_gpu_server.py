"""The served stream on the GPU: requests arriving while others run are
admitted between step groups and overlap on the device; every result must
be bit-identical to the same request solved alone, to the CPU oracle run of
the same request, and -- for a Helmholtz-array request and a sealed box with
a Debye region built as the stream builds them -- to the reference's own
outputs (tests/golden).  Tolerance: none."""
import numpy as np
import pytest

import cases as C
from conftest import golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402
from strata_fdtd_gb300.server import GPUExecutor, Request, SolveServer, solve_bytes  # noqa: E402
from strata_fdtd_gb300.workloads import served_stream  # noqa: E402
from oracle import oracle as O  # noqa: E402

from test_gpu_parity import API  # noqa: E402


def _oracle_twin(s, courant=0.5):
    """The same solve on the CPU oracle, from the GPU solver's set-up: mask,
    PML depth, materials and their ids, point sources, probes."""
    o = O.FDTDSolver(shape=s.shape, resolution=s.dx, c=s.c, rho=s.rho, courant=courant)
    assert o.dt == s.dt
    for b in s._boundaries:
        o.add_boundary(O.PML(depth=b.depth))
    if s._geometry_set:
        o.set_geometry(s.geometry.copy())
    for mid, mat in s._materials.items():
        o.register_material(mat, material_id=mid)
    if s._materials:
        o._material_id[...] = s._material_id
    for src in s._sources:
        o.add_source(O.GaussianPulse(position=tuple(src.position), frequency=src.frequency,
                                     amplitude=src.amplitude))
    for name, pr in s._probes.items():
        o.add_probe(name, tuple(pr.position))
    return o


def test_served_requests_match_the_oracle_and_reference_goldens():
    """Six requests of the stream's mix (free field, sealed box, Helmholtz
    block, Debye regions) arriving together with two requests built from the
    reference-pinned cases; all are admitted at once and run in shared
    batched step groups.  Every served trace equals the CPU oracle's run of
    the same request, and the two case requests equal the reference's
    traces, bit for bit."""
    mix = served_stream(seed=3, n_requests=6, rate=1e4, edges=(36, 64), steps=(80, 200),
                        pml=(4, 6), ade_fraction=0.6)
    cases = {"plain_served_helmholtz": C.PLAIN_CASES["served_helmholtz"],
             "ade_served_box_debye": C.ADE_CASES["served_box_debye"]}
    reqs = list(mix)
    for q, (key, case) in enumerate(cases.items()):
        reqs.append(Request(rid=100 + q, build=lambda case=case: C.build_case(API, case),
                            steps=case["steps"], arrival=0.0,
                            nbytes=solve_bytes(case["shape"], debye_poles=2),
                            cells=int(np.prod(case["shape"]))))
    srv = SolveServer(GPUExecutor(graph_steps=0), hbm_budget=160e9, step_group=64)
    stats = srv.run(reqs, realtime=False)
    assert stats["done"] == len(reqs), stats["errors"]
    assert stats["peak_active"] == len(reqs)
    results = {r.rid: r.result for r in srv.finished}
    kinds = set()
    for r in mix:
        s = r.build()
        o = _oracle_twin(s)
        o.run_steps(r.steps)
        kinds.add((bool(s._geometry_set), bool(s._materials)))
        for name, tr in o.get_probe_data().items():
            assert len(tr) == r.steps
            np.testing.assert_array_equal(results[r.rid][name], tr,
                                          err_msg=f"request {r.rid} probe {name}")
    assert len(kinds) >= 3, kinds  # free / solid / ADE requests all present
    for q, key in enumerate(cases):
        g = golden(key)
        for name in g["probe_names"]:
            np.testing.assert_array_equal(results[100 + q][str(name)], g[f"trace__{name}"],
                                          err_msg=f"{key} probe {name}")


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


def test_served_requests_with_the_wider_feature_set_match_goldens():
    """Requests using a nonuniform grid, microphones, Mur/radiation plane
    boundaries and membrane sources, served together (the batch steps the
    last two kinds through their own plans): each result equals the
    reference's probe traces."""
    keys = ["nu_regions_sdf", "mics_geom", "abc_all_sources", "membranes", "c1_tiny"]
    reqs = []
    for q, key in enumerate(keys):
        case = C.PLAIN_CASES[key]
        shape = case.get("shape") or (40, 40, 40)
        reqs.append(Request(rid=q, build=lambda case=case: C.build_case(API, case),
                            steps=case["steps"], arrival=0.0, nbytes=solve_bytes(shape),
                            cells=int(np.prod(shape))))
    srv = SolveServer(GPUExecutor(graph_steps=0), hbm_budget=160e9, step_group=48)
    stats = srv.run(reqs, realtime=False)
    assert stats["done"] == len(keys), stats["errors"]
    results = {r.rid: r.result for r in srv.finished}
    for q, key in enumerate(keys):
        g = golden("plain_" + key)
        for name in g["probe_names"]:
            np.testing.assert_array_equal(results[q][str(name)], g[f"trace__{name}"],
                                          err_msg=f"{key} probe {name}")


def test_background_server_serves_posts_from_threads():
    """The server in its background thread (start / post / wait / stop):
    requests posted from two client threads share step groups on the GPU
    and each result equals the request solved alone."""
    import threading
    import time

    reqs = served_stream(seed=13, n_requests=8, rate=1e4, edges=(36, 60), steps=(60, 160),
                         pml=(4, 6), ade_fraction=0.5)
    alone = served_stream(seed=13, n_requests=8, rate=1e4, edges=(36, 60), steps=(60, 160),
                          pml=(4, 6), ade_fraction=0.5)
    srv = SolveServer(GPUExecutor(), hbm_budget=160e9, step_group=32).start()

    def client(part):
        for r in part:
            srv.post(r)
            time.sleep(0.01)

    threads = [threading.Thread(target=client, args=(reqs[k::2],)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for r in reqs:
        assert r.wait(120), r.rid
    stats = srv.stop()
    assert stats["done"] == 8, stats["errors"]
    assert stats["peak_active"] > 1
    for r, a in zip(reqs, alone):
        s = a.build()
        s.run_steps(a.steps)
        for name, tr in s.get_probe_data().items():
            np.testing.assert_array_equal(r.result[name], tr, err_msg=f"request {r.rid}")
