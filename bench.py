#!/usr/bin/env python3
"""Benchmark: the 400^3 enclosure solve (strata-fdtd time-step path) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one GPU per rank, replicas only -- the path does not shard): 400^3
uniform grid, 1 mm cells, air, PML 16, rigid walls voxelised from the box
enclosure with its port, 2 kHz pulse, 8 probes (strata_fdtd_gb300.workloads).
One bench step = ``--inner`` (default 100) FDTD time steps; the default
K = 40 covers the workload's 4000 steps.

Metric: Gcell-updates/s (cells x time steps / s), whole job (sum over ranks
/ max-over-ranks time).  ``value`` is device-timed with inputs resident in
HBM (the 1.1 GB state is larger than L2, so no flush is needed); ``e2e`` is
the same metric through the public API with host-resident (pinned) fields
uploaded and the pressure field and probe traces read back every bench step.
``roofline`` relates the fused step kernel to HBM bandwidth (33 algorithmic
bytes per cell-update: 16 read + 16 written for p, vx, vy, vz, plus the 1-byte
cell-flag read); ``cpu_baseline`` is the CPU oracle (the bit-exact C
restatement of the reference native kernels, OpenMP) on a bounded sample.

--impl reference times that CPU implementation alone (all host threads) on
the same workload and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CELLS = 400 ** 3
BYTES_PER_CELL = 33
METRIC = "Gcell-updates/s"
WORKLOAD = "enclosure_400: 400^3 uniform 1 mm, PML 16, box enclosure 200x120x300 mm (12 mm walls, r25x80 mm port), 2 kHz pulse, 8 probes, 4000 steps"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--inner", type=int, default=100, help="FDTD time steps per bench step")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--size", type=int, default=400, help="grid edge (400 = the workload)")
    ap.add_argument("--kernel", default="auto", help="auto (autotuned) or a kernel configuration name")
    ap.add_argument("--ichunk", type=int, default=0, help="planes per block (march)")
    ap.add_argument("--workload", default="enclosure",
                    choices=["enclosure", "batch", "serve", "adjoint"])
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--requests", type=int, default=1000)
    ap.add_argument("--step-group", type=int, default=250)
    ap.add_argument("--max-active-cells", type=int, default=1 << 28,
                    help="served stream: cap on the cells of the running solves (0 = none)")
    ap.add_argument("--solo-cells", type=int, default=1 << 24,
                    help="served stream: solves this large step alone (0 = batch all)")
    ap.add_argument("--serve-graph-steps", type=int, default=50,
                    help="served stream: CUDA-graph replay length of each batched group (0 = none)")
    ap.add_argument("--batch-min-cells", type=int, default=0,
                    help="served stream: groups with fewer batchable cells step one by one")
    ap.add_argument("--serve-only", action="store_true",
                    help="served stream: skip the one-at-a-time arm (tuning runs)")
    ap.add_argument("--batch-solves", type=int, default=64)
    ap.add_argument("--batch-config", default="auto",
                    help="batch: auto (autotuned) or kernel:ROWSxICHUNK, e.g. column:16x16")
    ap.add_argument("--batch-of-one", action="store_true",
                    help="batch: also time each solve alone as a batch of one (same tile kernel)")
    ap.add_argument("--batch-only", action="store_true",
                    help="batch: skip the sequential baselines (profiling runs)")
    ap.add_argument("--graph-steps", type=int, default=50)
    ap.add_argument("--no-extras", action="store_true",
                    help="enclosure line only: skip the batched, served, adjoint and parity "
                         "sub-objects")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(x: float, dist, device: str) -> float:
    """The slowest rank's time: every rank's replica must finish."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, cell_updates_per_rank: int, seconds: float) -> float:
    """Whole-job Gcell-updates/s of `world` replicas that each did the same
    work in (at most) `seconds`: weak scaling, no collective on the data path."""
    return world * cell_updates_per_rank / seconds / 1e9


def profiled_traffic():
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_step_enclosure_400.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch_400:"):
                return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_id), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def smi_id(torch, local):
    """The nvidia-smi id (UUID) of the CUDA device ``local`` of this process."""
    try:
        u = str(torch.cuda.get_device_properties(local).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
        return cvd.split(",")[local] if cvd else str(local)


def oracle_enclosure(geometry):
    """The workload on the CPU oracle (float, reference native semantics)."""
    from oracle import oracle as O
    from strata_fdtd_gb300.workloads import enclosure_probes

    o = O.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    o.add_boundary(O.PML(depth=16))
    o.set_geometry(geometry)
    o.add_source(O.GaussianPulse(position=(200, 200, 200), frequency=2000.0))
    for q, pos in enumerate(enclosure_probes(geometry)):
        o.add_probe(f"probe{q}", pos)
    return o


def oracle_geometry():
    """Enclosure mask from the oracle's NumPy SDF restatement, in i-slabs."""
    from oracle import oracle as O

    c = (0.2, 0.2, 0.2)
    solid = O.Difference(O.Box(center=c, size=(0.2, 0.12, 0.3)),
                         O.Box(center=c, size=(0.176, 0.096, 0.276)),
                         O.Cylinder(p1=(0.2, 0.2, 0.05), p2=(0.2, 0.2, 0.13), radius=0.025))
    g = O.UniformGrid((400, 400, 400), 1e-3)
    out = np.empty((400, 400, 400), dtype=bool)
    Y, Z = np.meshgrid(g.y_coords, g.z_coords, indexing="ij")
    for i0 in range(0, 400, 25):
        xs = g.x_coords[i0:i0 + 25]
        X = np.repeat(xs, Y.size)
        pts = np.stack([X, np.tile(Y.ravel(), len(xs)), np.tile(Z.ravel(), len(xs))], axis=1)
        out[i0:i0 + 25] = (solid.sdf(pts) <= 0).reshape(len(xs), 400, 400)
    return ~out


def time_oracle(o, seconds):
    """Run the oracle for about ``seconds``; returns (Gcell/s, steps, threads)."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    o.run_steps(2)
    per = (time.perf_counter() - t0) / 2
    n = max(2, int(seconds / max(per, 1e-6)))
    t0 = time.perf_counter()
    o.run_steps(n)
    dt = time.perf_counter() - t0
    return CELLS * n / dt / 1e9, n, O.threads()


def workload_config(world):
    """The ``config`` object of both arms' lines: the workload and how it is
    spread over the ranks (one full replica per rank)."""
    return {"workload": WORKLOAD, "global_batch": world, "parallelism": f"replicas x{world}",
            "l2": "state 1.1 GB per replica > 129 MB L2, no flush"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    geometry = oracle_geometry()
    o = oracle_enclosure(geometry)
    inner = 2
    for _ in range(args.warmup):
        o.run_steps(inner)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run_steps(inner)
    el = time.perf_counter() - t0
    v = CELLS * inner * args.steps / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.gpus),
        "bench_step": f"{inner} FDTD steps on the CPU (rank 0)",
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": O.threads(), "kind": "port",
                         "sample": f"{inner * args.steps} FDTD steps of the 400^3 enclosure "
                                   "workload (oracle/sf_oracle.c, bit-exact restatement of the "
                                   "reference native kernels; OpenMP)"},
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch

    import strata_fdtd_gb300 as S
    from strata_fdtd_gb300 import _native
    from strata_fdtd_gb300.workloads import enclosure

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    lib = _native.load()
    n_edge = args.size
    cells = n_edge ** 3
    s = enclosure(n_edge)
    tune = None
    if args.kernel == "auto":
        s.set_kernel("auto", args.ichunk)
        tune = s.autotune(launches=10)  # times each configuration; state unchanged
        chosen = tune["best"]
    else:
        s.set_kernel(args.kernel, args.ichunk)
        chosen = args.kernel
    inner, K, W = args.inner, args.steps, args.warmup
    n_src = len(s._sources)
    n_probe = len(s._probes)
    # device-resident inputs for every timed step: waveform table and trace buffer
    s._sync_tables()
    s._upload_exposed()
    total = (W + K) * inner
    vals = torch.from_numpy(s._source_values(total)).to("cuda")
    trace = torch.empty((total, n_probe), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def bench_step(q):
        rc = lib.sf_plan_step(s._plan, inner, vals.data_ptr() + q * inner * n_src * 8,
                              trace.data_ptr() + q * inner * n_probe * 4, stream.cuda_stream)
        _native.check(rc, "sf_plan_step")

    for q in range(W):
        bench_step(q)
    barrier()
    clocks = ClockSampler(smi_id(torch, local))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for q in range(W, W + K):
        bench_step(q)
    end.record(stream)
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(start.elapsed_time(end), dist, "cuda")
    # per bench step: the step kernels, and one probe gather per sf_plan_step
    # call or captured block of steps (run_steps replays 50-step graphs)
    G = S.FDTDSolver._GRAPH_STEPS if s._kernel_auto else inner + 1
    launches = K * (inner + inner // G + (1 if inner % G else 0))
    value = replica_rate(world, cells * inner * K, ms / 1e3)
    kernel_ms = ms / (K * inner)  # every timed launch attributed to the step kernel
    hbm, peak_kind = peaks()
    achieved = BYTES_PER_CELL * cells / (kernel_ms / 1e3) / 1e9
    traffic = profiled_traffic()
    s._mark_device_newer()
    s._step_count += (W + K) * inner

    # end to end through the public API: pinned host fields in, p and traces out
    e2e = None
    if not args.no_e2e:
        host = {f: torch.zeros((n_edge,) * 3, dtype=torch.float32).pin_memory().numpy()
                for f in ("p", "vx", "vy", "vz")}
        for f in host:
            np.copyto(host[f], getattr(s, f))
        Ke = max(4, min(K, 10))
        # (a) one replica, each bench step's copies in line with its steps
        barrier()
        t0 = time.perf_counter()
        for _ in range(Ke):
            for f in host:
                setattr(s, f, host[f])
            s.run_steps(inner)
            _ = s.p
            _ = s.get_probe_data()
        torch.cuda.synchronize()
        el_serial = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
        # (b) two replicas of the workload alternate: bench step k loads its
        # four fields from pinned host memory into one replica and reads back
        # its p and probe traces on a copy stream, while the other replica
        # steps bench step k - 1 on the compute stream
        s2 = enclosure(n_edge)
        if args.kernel == "auto":
            s2.set_kernel("auto", args.ichunk)
            s2.autotune(launches=10)
        else:
            s2.set_kernel(args.kernel, args.ichunk)
        reps = (s, s2)
        outs = [{"p": torch.empty((n_edge,) * 3, dtype=torch.float32).pin_memory().numpy()}
                for _ in reps]
        comp, cp = torch.cuda.current_stream(), torch.cuda.Stream()

        def pipelined(jobs):
            ran, pend = [None, None], []
            up = torch.cuda.Event()
            with torch.cuda.stream(cp):
                reps[0].load_fields_async(**host)
                up.record(cp)
            for k in range(jobs):
                a = reps[k % 2]
                comp.wait_event(up)
                a.run_steps(inner)
                ran[k % 2] = torch.cuda.Event()
                ran[k % 2].record(comp)
                with torch.cuda.stream(cp):
                    if k + 1 < jobs:
                        if ran[(k + 1) % 2] is not None:
                            cp.wait_event(ran[(k + 1) % 2])  # that replica's last steps
                        reps[(k + 1) % 2].load_fields_async(**host)
                        up = torch.cuda.Event()
                        up.record(cp)
                    cp.wait_event(ran[k % 2])
                    pend.append((a.fields_async(("p",), out=outs[k % 2]), a.probe_data_async()))
                if len(pend) == 2:  # bench step k - 1's results, read on the host
                    fp, ft = pend.pop(0)
                    fp(), ft()
            for fp, ft in pend:
                fp(), ft()

        pipelined(2)  # untimed: the second replica's first use
        barrier()
        t0 = time.perf_counter()
        pipelined(Ke)
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
        del s2, reps
        e2e = {"value": replica_rate(world, cells * inner * Ke, el), "unit": METRIC,
               "h2d_bytes_per_step": 4 * cells * 4 + inner * n_src * 8,
               "d2h_bytes_per_step": cells * 4 + inner * n_probe * 4,
               "steps": Ke,
               "path": "two FDTDSolver replicas alternate: each bench step loads its four "
                       "fields from pinned host memory (load_fields_async) and reads back p "
                       "and the probe traces (fields_async, probe_data_async) on a copy "
                       "stream while the other replica runs run_steps(inner); every result "
                       "is read on the host",
               "serial_value": replica_rate(world, cells * inner * Ke, el_serial),
               "serial_path": "one FDTDSolver: fields assigned from pinned host arrays, "
                              "run_steps(inner), solver.p and get_probe_data() read back, "
                              "in line"}

    def cpu_point():
        from oracle import oracle as O

        o = oracle_enclosure(s.geometry)
        v, n, th = time_oracle(o, args.cpu_seconds)
        # the single-thread point of the same sample
        O.set_threads(1)
        v1, n1, _ = time_oracle(o, min(5.0, args.cpu_seconds))
        O.set_threads(th)
        del o
        return {"value": v, "unit": METRIC, "cores": th, "kind": "port",
                "sample": f"{n} FDTD steps of the same 400^3 enclosure workload on the CPU "
                          "oracle (bit-exact C restatement of the reference native kernels, "
                          "OpenMP, all host threads)",
                "value_1_thread": v1, "sample_1_thread": f"{n1} FDTD steps, 1 thread"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and n_edge == 400:
        cpu = _guarded(cpu_point)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": (workload_config(world) if n_edge == 400 else
                       {"workload": f"enclosure at {n_edge}^3", "global_batch": world,
                        "parallelism": f"replicas x{world}"}),
            "bench_step": f"{inner} FDTD time steps",
            "kernel": {"name": chosen, "i_chunk": args.ichunk, "autotune_ms_per_step": tune},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                         "bytes_per_cell": BYTES_PER_CELL,
                         "kernel": f"fused step kernel, configuration {chosen}"},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "device": torch.cuda.get_device_name(local),
            "library": lib.sf_version().decode(),
        }
        if world == 1 and not args.no_extras and n_edge == 400:
            del s, vals, trace
            torch.cuda.empty_cache()
            line.update(extras(args))
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def parity_quick_start():
    """The 100^3 quick start, 1000 steps on the GPU through FDTDSolver.run_steps,
    against the CPU oracle: bit-exact in FP32, and its rel-L2 against the
    oracle's FP64 build."""
    from oracle import oracle as O
    from strata_fdtd_gb300.workloads import quick_start_100

    s = quick_start_100()
    s.run_steps(1000)
    gpu = {f: getattr(s, f) for f in ("p", "vx", "vy", "vz")}
    tr = s.get_probe_data()["output"]
    out = {"workload": "quick_start_100 (100^3, PML 10, 1 kHz, 1000 steps)"}
    for prec in ("f32", "f64"):
        o = O.FDTDSolver(shape=(100, 100, 100), resolution=1e-3, c=343.0, rho=1.204,
                         courant=0.5, precision=prec)
        o.add_boundary(O.PML(depth=10))
        o.add_source(O.GaussianPulse(position=(50, 50, 50), frequency=1000.0))
        o.add_probe("output", (75, 50, 50))
        o.run_steps(1000)
        ref = {f: getattr(o, f) for f in gpu}
        rt = o.get_probe_data()["output"]
        if prec == "f32":
            out["bit_exact_vs_oracle_f32"] = bool(
                all(np.array_equal(gpu[f], ref[f]) for f in gpu) and np.array_equal(tr, rt))
        else:
            for f in gpu:
                out[f"rel_l2_{f}_vs_f64"] = float(
                    np.linalg.norm(gpu[f].astype(np.float64) - ref[f]) / np.linalg.norm(ref[f]))
            out["rel_l2_trace_vs_f64"] = float(
                np.linalg.norm(tr.astype(np.float64) - rt) / np.linalg.norm(rt))
    return out


# The 400^3 enclosure over all 4000 steps is checked by
# tests/test_gpu_workloads_full.py (about 5 minutes of CPU oracle time, too
# long for this benchmark): bit-exact against the FP32 oracle, and these
# rel-L2 errors against the FP64 oracle, measured on a GB300 machine.
ENCLOSURE_FP64_ERRORS = {
    "workload": "enclosure_400, 4000 steps (recorded by tests/test_gpu_workloads_full.py)",
    "bit_exact_vs_oracle_f32": True, "rel_l2_p_vs_f64": 3.29e-6, "rel_l2_vx_vs_f64": 2.48e-6,
    "rel_l2_vy_vs_f64": 3.08e-6, "rel_l2_vz_vs_f64": 3.34e-6, "rel_l2_traces_vs_f64": 1.51e-6,
}


def _guarded(fn):
    """fn() or, if it raises, {"error": ...} with the traceback on stderr:
    a failing part leaves the rest of the line, the headline included."""
    import traceback

    try:
        return fn()
    except Exception as e:  # noqa: BLE001
        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"}


def _batched_part(args):
    b = run_batch(args)
    return {
        "value": b["value"], "unit": b["unit"], "workload": b["config"]["workload"],
        "cell_updates": b["config"]["cell_updates"],
        "sequential_value": (b["sequential"] or {}).get("value"),
        "speedup_vs_sequential": b["speedup_vs_sequential"],
        "traces_identical": b["traces_identical"], "plain_kernel": b["config"]["plain_kernel"],
        "rejected_materials": b["config"]["rejected_materials"],
        "cpu_baseline": b.get("cpu_baseline")}


def _served_part(args):
    sv = run_serve(args)
    return {
        "value": sv["value"], "unit": sv["unit"], "workload": sv["config"]["workload"],
        "p50_latency_s": sv["served"]["p50_latency_s"],
        "p99_latency_s": sv["served"]["p99_latency_s"],
        "makespan_s": sv["served"]["makespan_s"],
        "sequential_value": (sv["sequential"] or {}).get("gcell_updates_per_s"),
        "sequential_p50_latency_s": (sv["sequential"] or {}).get("p50_latency_s"),
        "sequential_p99_latency_s": (sv["sequential"] or {}).get("p99_latency_s"),
        "throughput_ratio": sv["throughput_ratio"], "results_identical": sv["results_identical"],
        "done": sv["served"]["done"], "peak_active": sv["served"]["peak_active"],
        "max_active_cells": args.max_active_cells, "cpu_baseline": sv.get("cpu_baseline")}


def _adjoint_part(args):
    a = run_adjoint(args)
    return {"value": a["value"], "unit": a["unit"], "workload": a["config"]["workload"],
            "accuracy": a["config"]["accuracy"],
            **{k: {q: a[k][q] for q in ("gradient_seconds", "forward_seconds",
                                         "gradient_gcell_updates_per_s")}
               for k in ("dw", "f32", "f64")}}


def extras(args):
    """The second half of the metric on the same GPU, each on its configured
    workload: the batched heterogeneous launch, the served request stream
    (p50/p99 beside throughput, against one request at a time) and the
    differentiable solve, plus the parity record.  Each part is guarded, so
    one that fails is reported as an error beside the others."""
    import torch

    out = {}
    for key, part in (("batched", _batched_part), ("served", _served_part),
                      ("adjoint", _adjoint_part)):
        out[key] = _guarded(lambda: part(args))
        torch.cuda.empty_cache()
    out["parity"] = {"quick_start_100": _guarded(parity_quick_start),
                     "enclosure_400": ENCLOSURE_FP64_ERRORS}
    return out


def oracle_twin(s):
    """The same solve on the CPU oracle, built from a GPU solver's set-up:
    mask, PML depth, ADE materials and their ids, point sources, probes."""
    from oracle import oracle as O

    o = O.FDTDSolver(shape=s.shape, resolution=s.dx, c=s.c, rho=s.rho, courant=0.5)
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


def cpu_subsample(solvers, steps_each, full_cell_updates, what):
    """The CPU baseline of a many-solve workload: the oracle (all host
    threads) runs ``steps_each`` steps of each solve of a seeded subsample,
    after one untimed step; the rate is cell-updates over the summed time,
    and the whole workload's CPU time is extrapolated from it by
    cell-updates."""
    from oracle import oracle as O

    el, cu = 0.0, 0
    for s in solvers:
        o = oracle_twin(s)
        o.run_steps(1)
        t0 = time.perf_counter()
        o.run_steps(steps_each)
        el += time.perf_counter() - t0
        cu += int(np.prod(s.shape)) * steps_each
        del o
    v = cu / el / 1e9
    return {"value": v, "unit": METRIC, "cores": O.threads(), "kind": "port",
            "sample": f"{steps_each} steps of each of {what} on the CPU oracle (bit-exact C "
                      "restatement of the reference native kernels and its ADE kernels, OpenMP), "
                      f"{cu / 1e9:.3f} G cell-updates in {el:.2f} s; the whole workload "
                      "extrapolated by cell-updates",
            "full_workload_seconds_estimate": full_cell_updates / (v * 1e9)}


def run_batch(args):
    """The heterogeneous batch: 64 grids (edges 64-256), solids, a 2-pole
    Debye block each, 500-3000 steps; batched persistent launches under CUDA
    graphs vs the same solves one after another through the single-grid path.
    Both produce bit-identical results (tests/test_gpu_batch.py)."""
    import torch

    from strata_fdtd_gb300.batch import BatchedSolver
    from strata_fdtd_gb300.workloads import batch_workload

    n = args.batch_solves
    seq, steps, info = batch_workload(seed=0, n_solves=n)
    cell_updates = sum(int(np.prod(s.shape)) * q for s, q in zip(seq, steps))
    # untimed warm-up of every path the arms use (CUDA modules, torch kernels,
    # a padded twin, a batch with graphs), so no arm pays the first-use costs
    warm, wsteps, _ = batch_workload(seed=1, n_solves=2)
    for w in warm:
        w.run_steps(40)
    BatchedSolver(warm).run_steps(60, graph_steps=args.graph_steps)
    del warm
    torch.cuda.synchronize()
    t_seq = t_one = float("nan")
    traces_seq = None
    if not args.batch_only:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s, q in zip(seq, steps):
            s.run_steps(q)
        torch.cuda.synchronize()
        t_seq = time.perf_counter() - t0
        traces_seq = [s.get_probe_data() for s in seq]
    del seq
    torch.cuda.empty_cache()
    if args.batch_of_one and not args.batch_only:
        # second baseline: each solve alone through the batch tile kernel (a batch of one)
        one, _, _ = batch_workload(seed=0, n_solves=n)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s, q in zip(one, steps):
            BatchedSolver([s]).run_steps(q, graph_steps=args.graph_steps)
        torch.cuda.synchronize()
        t_one = time.perf_counter() - t0
        del one
        torch.cuda.empty_cache()
    bat, _, _ = batch_workload(seed=0, n_solves=n)
    b = BatchedSolver(bat)
    if args.batch_config == "auto":
        tune = b.autotune(launches=2)
    else:
        kernel, shape = args.batch_config.split(":")
        rows, ich = (int(v) for v in shape.split("x"))
        b.kernel, b.rows, b.i_chunk = kernel, rows, ich
        tune = {}
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    start.record()
    b.run_steps(steps, graph_steps=args.graph_steps)
    end.record()
    torch.cuda.synchronize()
    t_bat_wall = time.perf_counter() - t0
    t_bat = start.elapsed_time(end) / 1e3
    same = traces_seq is not None and all(
        all(np.array_equal(bs.get_probe_data()[k], tr[k]) for k in tr)
        for bs, tr in zip(bat, traces_seq))
    line = {
        "metric": "Gcell-updates/s (batched uneven grids)", "value": cell_updates / t_bat / 1e9,
        "unit": "Gcell-updates/s", "n_gpus": 1, "steps": int(max(steps)), "warmup": 0,
        "ms_per_step": t_bat / max(steps) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batch of {n} grids, edges log-U[64,256], PML 8, 1-6 solids, "
                               "2-pole Debye block, 1-4 kHz pulse, 2 probes, 500-3000 steps",
                   "cells": int(sum(np.prod(s.shape) for s in bat)),
                   "cell_updates": cell_updates, "plain_kernel": b.kernel, "tile_rows": b.rows,
                   "i_chunk": b.i_chunk,
                   "graph_steps": args.graph_steps, "rejected_materials": info["rejected_materials"],
                   "autotune_ms_per_step": {f"{k[0]}:{k[1]}x{k[2]}": v for k, v in tune.items()
                                            if k != "best"}},
        "sequential": None if t_seq != t_seq else {
            "value": cell_updates / t_seq / 1e9, "seconds": t_seq,
            "path": "each solve alone through FDTDSolver.run_steps"},
        "sequential_tile_kernel": None if t_one != t_one else {
            "value": cell_updates / t_one / 1e9, "seconds": t_one,
            "path": "each solve alone as a batch of one (same tile kernel)"},
        "speedup_vs_sequential_tile_kernel": None if t_one != t_one else t_one / t_bat,
        "batched_wall_seconds": t_bat_wall,
        "speedup_vs_sequential": None if t_seq != t_seq else t_seq / t_bat,
        "traces_identical": bool(same),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_subsample(bat[:16], 60, cell_updates,
                                             "the first 16 solves of the batch")
    return line


def run_serve(args):
    """The served stream: Poisson arrivals at 200/s, edges 48-320, 500-5000
    steps, mixed geometry, optional Debye region, 160 GB budget; continuous
    batching vs one solve at a time on the same GPU, same requests."""
    import torch

    from strata_fdtd_gb300.server import GPUExecutor, SequentialExecutor, SolveServer
    from strata_fdtd_gb300.workloads import served_stream

    n = args.requests
    ex = GPUExecutor(graph_steps=args.serve_graph_steps, solo_cells=args.solo_cells or None,
                     batch_min_cells=args.batch_min_cells)
    srv = SolveServer(ex, hbm_budget=160e9, step_group=args.step_group,
                      max_active_cells=args.max_active_cells or None)
    st = srv.run(served_stream(seed=0, n_requests=n), realtime=True)
    st["host_advance_s"], st["host_wait_s"] = ex.host_advance_s, ex.host_wait_s
    st["host_build_s"] = ex.host_build_s
    st["host_s"] = {k: round(v, 2) for k, v in ex.host_s.items()}
    res = {r.rid: r.result for r in srv.finished if r.status == "done"}
    del srv
    torch.cuda.empty_cache()
    st2, same = {"gcell_updates_per_s": None}, None
    if not args.serve_only:
        ex2 = SequentialExecutor()
        seq = SolveServer(ex2, hbm_budget=160e9, step_group=10**9, max_active=1)
        st2 = seq.run(served_stream(seed=0, n_requests=n), realtime=True)
        st2["host_advance_s"], st2["host_wait_s"] = ex2.host_advance_s, ex2.host_wait_s
        st2["host_build_s"] = ex2.host_build_s
        same = bool(all(all(np.array_equal(res[r.rid][k], r.result[k]) for k in r.result)
                        for r in seq.finished if r.status == "done" and r.rid in res))
    line = {
        "metric": "Gcell-updates/s (served stream)", "value": st["gcell_updates_per_s"],
        "unit": "Gcell-updates/s", "n_gpus": 1, "steps": st["step_groups"], "warmup": 0,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n} requests, Poisson 200/s, edges log-U[48,320], steps "
                               "U[500,5000], PML 8-16, free/box/Helmholtz-array geometry, "
                               "50% with a 1-2 pole Debye region, 160 GB budget",
                   "step_group": args.step_group, "max_active_cells": args.max_active_cells,
                   "solo_cells": args.solo_cells, "graph_steps": args.serve_graph_steps,
                   "batch_min_cells": args.batch_min_cells},
        "served": st, "sequential": st2,
        "throughput_ratio": ((st["gcell_updates_per_s"] or 0) / st2["gcell_updates_per_s"]
                             if st2["gcell_updates_per_s"] else None),
        "results_identical": same,
    }
    if not args.no_cpu_baseline:
        sub = [r.build() for r in served_stream(seed=0, n_requests=20)]
        line["cpu_baseline"] = cpu_subsample(sub, 50, st.get("cell_updates") or 0,
                                             "the first 20 requests of the stream")
        del sub
        torch.cuda.empty_cache()
    return line


def run_adjoint(args):
    """The differentiable solve: 128^3, 10-cell PML, design field on the
    central 64^3, 1.5 kHz source, two probes, 2000 steps, checkpoints every
    100 steps.  Times one probe-loss gradient (forward with checkpoints,
    segment recomputation, reverse-time adjoint, dL/dtheta) against the
    forward alone, in FP32 and FP64 working precision."""
    import torch

    from strata_fdtd_gb300.adjoint import DifferentiableSolver
    from strata_fdtd_gb300.workloads import design_field

    shape, n = (128, 128, 128), args.adjoint_steps
    cells = int(np.prod(shape))
    probes = [(100, 64, 64), (64, 100, 40)]
    out = {}
    for name, dt in (("dw", "dw"), ("f32", torch.float32), ("f64", torch.float64)):
        s = DifferentiableSolver(shape, pml_depth=10, frequency=1500.0, source=(30, 64, 64),
                                 probes=probes, dtype=dt, checkpoint_every=100)
        theta = torch.tensor(design_field(shape, 64, seed=0), device="cuda", dtype=s.ext_dtype)
        target = s.forward(torch.tensor(design_field(shape, 64, seed=1), device="cuda"), n)[0]
        th = theta.clone().requires_grad_(True)
        w = min(200, n)
        s.loss(th, target[:w], w).backward()  # warm-up
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        s.forward(theta, n, keep_checkpoints=False)
        e1.record()
        th = theta.clone().requires_grad_(True)
        s.loss(th, target, n).backward()
        e2.record()
        torch.cuda.synchronize()
        t_fwd, t_grad = e0.elapsed_time(e1) / 1e3, e1.elapsed_time(e2) / 1e3
        out[name] = {"gradient_seconds": t_grad, "forward_seconds": t_fwd,
                     "gradient_over_forward": t_grad / t_fwd,
                     "forward_gcell_updates_per_s": cells * n / t_fwd / 1e9,
                     "gradient_gcell_updates_per_s": cells * n / t_grad / 1e9,
                     "peak_device_bytes": int(torch.cuda.max_memory_allocated())}
        del s, theta, target, th
        torch.cuda.empty_cache()
    line = {"metric": "Gcell-updates/s (probe-loss gradient, forward steps per second)",
            "value": out["dw"]["gradient_gcell_updates_per_s"], "unit": "Gcell-updates/s",
            "n_gpus": 1, "steps": n, "warmup": 1, "ms_per_step": out["dw"]["gradient_seconds"] / n * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32x2 (double-word)", "data": "synthetic",
            "config": {"workload": f"128^3, PML 10, design field on the central 64^3, 1.5 kHz "
                                   f"source, 2 probes, {n} steps, checkpoints every 100 steps",
                       "accuracy": "double-word and FP64 gradients within 1.2e-6 of FP64 central "
                                   "differences per sampled cell, FP32 within 8.2e-4 "
                                   "(tests/test_gpu_adjoint.py)"},
            "dw": out["dw"], "f32": out["f32"], "f64": out["f64"]}
    return line


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        print(json.dumps(run_batch(args)))
    elif args.workload == "serve":
        print(json.dumps(run_serve(args)))
    elif args.workload == "adjoint":
        print(json.dumps(run_adjoint(args)))
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
