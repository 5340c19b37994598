"""GPU parity of the multi-step pipeline kernels (k_step_pipe): several
steps per launch through rings of planes kept in L2, against the CPU oracle
and against single steps, bit for bit.

Covered: every pipeline configuration, planes per chunk from 1 to past nx,
step counts that leave single steps over, several calls in a row, probes
on chunk and tile edges (their traces include the intermediate states),
point and plane sources, geometry, PML, nonuniform grids, the autotuner's
choice, and the 400^3 enclosure against the single-step kernel.
"""
import numpy as np
import pytest

import cases as C
from conftest import sha256

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

from test_gpu_parity import API  # noqa: E402

ORACLE = O.make_api()
PIPES = [c for c in S.solver.kernel_configs() if c.startswith(("tile_pipe", "tile_stream"))]


def _case(shape, steps, geometry=True):
    nx, ny, nz = shape

    def at(i, j, k):
        return (min(i, nx - 1), min(j, ny - 1), min(k, nz - 1))

    case = dict(shape=shape, res=1e-3, courant=0.6, pml=dict(depth=3 if min(shape) >= 8 else 1),
                sources=[("point", (nx // 2, ny // 3, nz // 4), 25000.0, 1.0),
                         ("point", (2, ny - 1, 4), 30000.0, 0.7),
                         ("plane", {"axis": 0, "index": nx - 3}, 9000.0, 0.2),
                         ("plane", {"axis": 2, "index": min(nz - 1, 33)}, 15000.0, 0.25)],
                probes=[("a", (nx // 2, ny // 2, nz // 2)), ("b", (0, 0, 0)),
                        ("c", (nx - 1, ny - 1, nz - 1)), ("d", at(4, 15, 31)), ("e", at(5, 16, 32))],
                steps=steps)
    if geometry:
        case["geometry"] = dict(kind="blocks", seed=sum(shape), n_boxes=2, n_spheres=1)
    return case


def _check(s, ref, tag):
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"{tag} {f}")
    for name in ref.get_probe_data():
        np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name],
                                      err_msg=f"{tag} probe {name}")


@pytest.mark.parametrize("config", PIPES)
@pytest.mark.parametrize("shape,S", [((23, 37, 64), 0), ((23, 37, 64), 1), ((17, 20, 36), 3),
                                     ((9, 33, 40), 4), ((6, 5, 8), 2), ((12, 70, 132), 5),
                                     ((10, 17, 44), 40)])
def test_pipeline_against_oracle(config, shape, S):
    """Calls of 1, 7 and 12 steps: every pipeline launch and the single
    steps left over, with probes and sources on chunk and tile edges."""
    case = _case(shape, 20, geometry=min(shape) >= 8)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(20)
    s = C.build_case(API, case)
    s.set_kernel(config, S)
    for n in (1, 7, 12):
        s.run_steps(n)
    _check(s, ref, f"{config} {shape} S={S}")


@pytest.mark.parametrize("config", PIPES)
def test_pipeline_nonuniform_grid(config):
    g_args = ((26, 30, 36), 1e-3, 1.04, 1.0, 1.06)
    ref = ORACLE.FDTDSolver(grid=ORACLE.NonuniformGrid.from_stretch(*g_args), c=343.0, rho=1.204,
                            courant=0.5)
    s = S.FDTDSolver(grid=S.NonuniformGrid.from_stretch(*g_args), c=343.0, rho=1.204, courant=0.5)
    for x in (ref, s):
        x.add_boundary((O.PML if x is ref else S.PML)(depth=4))
        x.add_source((O.GaussianPulse if x is ref else S.GaussianPulse)(
            position=(13, 14, 18), frequency=20000.0))
        x.add_probe("m", (12, 15, 17))
    ref.run_steps(30)
    s.set_kernel(config, 3)
    s.run_steps(13)
    s.run_steps(17)
    _check(s, ref, config)


def test_autotune_skips_pipelines_and_stays_exact():
    """The autotuner times single-step configurations only (the pipelines
    run when chosen explicitly); a pipeline chosen after it still runs
    bit-exact from the tuned state."""
    case = _case((40, 64, 64), 30)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(30)
    s = C.build_case(API, case)
    ms = s.autotune(launches=3)
    assert not any(c in ms for c in PIPES) and ms["best"] not in PIPES, ms
    s.run_steps(11)
    s.set_kernel(PIPES[0])
    s.run_steps(19)
    _check(s, ref, f"autotuned {ms['best']}, then {PIPES[0]}")


@pytest.mark.parametrize("config", ["tile_pipe2_w4", "tile_stream2_w4"])
def test_pipeline_full_size_matches_single_steps(config):
    """The 400^3 enclosure from a random state: 10 pipelined steps equal 10
    single steps of the warp-tile kernel, fields and probe traces."""
    solid = C.c2_solid(API)
    rng = np.random.default_rng(11)
    runs = []
    for kernel in ("tile_r1_w4_m6", config):
        s = S.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
        s.add_boundary(S.PML(depth=16))
        s.set_geometry_sdf(solid)
        s.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0))
        for q, pos in enumerate(((200, 200, 230), (0, 0, 0), (399, 399, 399), (101, 127, 31))):
            s.add_probe(f"p{q}", pos)
        if not runs:
            init = rng.standard_normal((400, 400, 400), dtype=np.float32) * np.float32(1e-3)
            init[~s.geometry] = 0.0
        s.p = init.copy()
        s.set_kernel(kernel)
        s.run_steps(10)
        runs.append(s)
    a, b = runs
    for f in ("p", "vx", "vy", "vz"):
        assert sha256(getattr(a, f)) == sha256(getattr(b, f)), f
    for name in a.get_probe_data():
        np.testing.assert_array_equal(a.get_probe_data()[name], b.get_probe_data()[name])


@pytest.mark.parametrize("config", PIPES)
def test_expired_wait_fails_cleanly_and_next_call_is_exact(config):
    """The pipelines' cross-warp waits are bounded.  With a short bound and
    the test hook that makes the first work item also wait on a device flag
    nothing sets, the wait runs out: the kernel raises its error flag, every
    other wait and claim returns, and sf_plan_step reports the expiry (no
    fault, no hang).  The next call, with the hook off, steps the restored
    state exactly like the oracle."""
    from strata_fdtd_gb300 import _native

    lib = _native.load()
    case = _case((23, 37, 64), 6)
    s = C.build_case(API, case)
    ref = C.build_case(ORACLE, case)
    s.set_kernel(config)
    s.run_steps(4)
    ref.run_steps(4)
    saved = {f: getattr(s, f).copy() for f in ("p", "vx", "vy", "vz")}
    _native.check(lib.sf_plan_set_wait_limit(s._plan, 2000, 1), "sf_plan_set_wait_limit")
    with pytest.raises(_native.NativeError, match="dependency wait expired"):
        s.run_steps(6)
    torch.cuda.synchronize()  # the context is intact
    _native.check(lib.sf_plan_set_wait_limit(s._plan, 0, 0), "sf_plan_set_wait_limit")
    for f, v in saved.items():
        setattr(s, f, v)
    s.run_steps(6)
    ref.run_steps(6)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f)
    for name, tr in ref.get_probe_data().items():
        np.testing.assert_array_equal(s.get_probe_data()[name], tr, err_msg=name)
