"""Times the reference's own CPU path beside the oracle, on the same workload
and the same host cores.  Test infrastructure: it runs only where the
reference tree is present (REF_ROOT) and its native module has been built by
``make -C oracle ref``.  It is never part of the product or the benchmark.

The reference side is its public ``FDTDSolver`` (core/solver.py:1507) with
``backend="native"``: ``step()`` (core/solver.py:2003-2077) driving its
compiled ``_kernels`` passes, built from its own sources with its own x86
flags (``-O3 -march=x86-64-v2``, _kernels/CMakeLists.txt:36-70).  The oracle
side is ``oracle.FDTDSolver`` on ``sf_oracle.c`` (one fused loop per step,
``-O3 -ffp-contract=off``).  Both run the 400^3 enclosure (PML 16, the box
enclosure with its port, 2 kHz pulse, 8 probes) for ``--steps`` steps after
two untimed ones, with OpenMP threads set by ``--threads``; after the timed
steps the two pressure fields are compared bit for bit.

    make -C oracle ref
    python oracle/time_reference.py --threads 8 --steps 10
    python oracle/time_reference.py --threads 1 --steps 2

Prints one JSON line: each side's Gcell-updates/s and the oracle's rate
over the reference's.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--steps", type=int, default=10)
    args = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(args.threads)

    import numpy as np

    # this folder is the package ``oracle``, not a path entry of its own
    sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    from bench import oracle_enclosure, oracle_geometry
    from make_golden import load_reference
    from oracle import oracle as O
    from strata_fdtd_gb300.workloads import enclosure_probes

    O.set_threads(args.threads)
    api = load_reference()
    geometry = oracle_geometry()
    cells = geometry.size

    ref = api.FDTDSolver(shape=geometry.shape, resolution=1e-3, c=343.0, rho=1.204,
                         courant=0.5, backend="native")
    ref.add_boundary(api.PML(depth=16))
    ref.set_geometry(geometry)
    ref.add_source(api.GaussianPulse(position=(200, 200, 200), frequency=2000.0))
    for q, pos in enumerate(enclosure_probes(geometry)):
        ref.add_probe(f"probe{q}", pos)
    orc = oracle_enclosure(geometry)

    def timed(step):
        step(2)
        t0 = time.perf_counter()
        step(args.steps)
        return cells * args.steps / (time.perf_counter() - t0) / 1e9

    def ref_steps(n):
        for _ in range(n):
            ref.step()

    v_ref = timed(ref_steps)
    v_orc = timed(orc.run_steps)
    same = bool(np.array_equal(np.asarray(ref.p), orc.p))
    print(json.dumps({
        "workload": "enclosure_400", "threads": args.threads, "steps": args.steps,
        "reference_gcells": v_ref, "oracle_gcells": v_orc, "oracle_over_reference": v_orc / v_ref,
        "pressure_bit_identical": same,
        "reference_native_threads": int(api.kernels.get_num_threads()),
    }))


if __name__ == "__main__":
    main()
