"""GPU parity of the two-step kernels (k_step_tb2): two time steps per pass
over the state with overlapped tiles, against the CPU oracle and against
single steps, bit for bit.

Covered: every two-step configuration, planes per chunk from 1 to past nx,
odd step counts (the last step runs single), several calls in a row, point
and plane sources on and next to tile and chunk edges (the level-1 halo
recomputes them), probes on tile edges (their level-1 samples come from the
owning block), solids, PML, grids smaller than one tile, and the 400^3
enclosure against the single-step warp-tile kernel.
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
TBS = [c for c in S.solver.kernel_configs() if c.startswith("tb2")]


def _case(shape, steps, geometry=True):
    nx, ny, nz = shape

    def at(i, j, k):
        return (max(0, min(i, nx - 1)), max(0, min(j, ny - 1)), max(0, min(k, nz - 1)))

    case = dict(shape=shape, res=1e-3, courant=0.6, pml=dict(depth=3 if min(shape) >= 8 else 1),
                sources=[("point", at(nx // 2, ny // 3, nz // 4), 25000.0, 1.0),
                         ("point", at(2, 8, 80), 30000.0, 0.7),     # tile corner (tj 8, tk 80)
                         ("point", at(nx - 2, 7, 79), 27000.0, -0.6),
                         ("point", at(3, 12, 64), 21000.0, 0.5),    # tile corner (tj 12, tk 64)
                         ("plane", {"axis": 1, "index": min(ny - 1, 16)}, 9000.0, 0.2),
                         ("plane", {"axis": 2, "index": min(nz - 1, 81)}, 15000.0, 0.25),
                         ("plane", {"axis": 0, "index": min(nx - 1, 4)}, 11000.0, 0.15)],
                probes=[("a", at(nx // 2, ny // 2, nz // 2)), ("b", (0, 0, 0)),
                        ("c", at(nx - 1, ny - 1, nz - 1)), ("d", at(4, 7, 79)),
                        ("e", at(5, 8, 80)), ("f", at(1, 16, 60)), ("g", at(nx - 1, 0, 59))],
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


@pytest.mark.parametrize("config", TBS)
@pytest.mark.parametrize("shape,ich", [((23, 37, 64), 0), ((23, 37, 64), 1), ((17, 20, 36), 3),
                                       ((9, 33, 40), 4), ((6, 5, 8), 2), ((12, 70, 170), 5),
                                       ((10, 17, 44), 40), ((31, 19, 83), 0), ((3, 90, 161), 2)])
def test_two_step_against_oracle(config, shape, ich):
    """Calls of 1, 7 and 12 steps: two-step launches and the single steps
    left over, with sources and probes on and beside tile edges."""
    case = _case(shape, 20, geometry=min(shape) >= 8)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(20)
    s = C.build_case(API, case)
    s.set_kernel(config, ich)
    for n in (1, 7, 12):
        s.run_steps(n)
    _check(s, ref, f"{config} {shape} ich={ich}")


@pytest.mark.parametrize("config", TBS[:2])
def test_two_step_free_field(config):
    """A free-field grid (no flag bytes), 100 steps in one call."""
    case = _case((40, 48, 96), 100, geometry=False)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(100)
    s = C.build_case(API, case)
    s.set_kernel(config, 0)
    s.run_steps(100)
    _check(s, ref, config)


def test_two_step_full_size_matches_single_steps():
    """The 400^3 enclosure from a random state: 10 two-step-kernel steps
    equal 10 single steps of the warp-tile kernel, fields and probe traces."""
    solid = C.c2_solid(API)
    rng = np.random.default_rng(11)
    runs = []
    for kernel in ("tile_r1_w4_m6", TBS[0]):
        s = S.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
        s.add_boundary(S.PML(depth=16))
        s.set_geometry_sdf(solid)
        s.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0))
        for q, pos in enumerate(((200, 200, 230), (0, 0, 0), (399, 399, 399), (101, 127, 31),
                                 (200, 8, 80), (201, 7, 79))):
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
