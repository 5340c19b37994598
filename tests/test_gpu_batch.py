"""Batched solves (sf_batch_*): every member of a heterogeneous batch must be
bit-identical to the same solve run alone, with and without CUDA graphs, and
the batch autotuner must leave the state untouched.  Tolerance: none."""
import types

import numpy as np
import pytest

import cases as C
from conftest import golden, sha256

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402
from strata_fdtd_gb300.batch import BatchedSolver  # noqa: E402
from strata_fdtd_gb300.workloads import batch_workload  # noqa: E402

API = types.SimpleNamespace(
    FDTDSolver=S.FDTDSolver, UniformGrid=S.UniformGrid, PML=S.PML, GaussianPulse=S.GaussianPulse,
    Box=S.Box, Sphere=S.Sphere, Cylinder=S.Cylinder, Union=S.Union, Intersection=S.Intersection,
    Difference=S.Difference, HelmholtzResonator=S.HelmholtzResonator, Pole=S.Pole,
    PoleType=S.PoleType, SimpleMaterial=S.SimpleMaterial, NonuniformGrid=S.NonuniformGrid,
    MaterializedGeometry=S.MaterializedGeometry,
    ABCFirstOrder=S.ABCFirstOrder, RadiationImpedance=S.RadiationImpedance,
    CircularMembraneSource=S.CircularMembraneSource,
    RectangularMembraneSource=S.RectangularMembraneSource)

MIX = [("plain", "c1_tiny"), ("plain", "blocks_odd"), ("plain", "plane_yz_geom"),
       ("plain", "impulse_default_coeffs"), ("ade", "debye_2pole"), ("ade", "lorentz_mixed_geom"),
       ("plain", "sdf_geometry"), ("plain", "plane_x_pml_x")]


def _case(kind, name):
    return (C.ADE_CASES if kind == "ade" else C.PLAIN_CASES)[name]


def _fields(s):
    return {f: getattr(s, f).copy() for f in ("p", "vx", "vy", "vz")}


WIDE_MIX = [("plain", "nu_stretch_blocks"), ("plain", "nu_regions_sdf"),
            ("plain", "nu_stretch_low_end"), ("plain", "mics_geom"),
            ("plain", "mics_directional"), ("plain", "abc_all_sources"),
            ("plain", "rad_pml_mix"), ("plain", "membranes"), ("ade", "nu_mixed_geom"),
            ("plain", "blocks_odd"), ("ade", "debye_2pole")]


@pytest.mark.parametrize("graph_steps", [0, 16])
def test_batch_of_the_wider_feature_set_matches_goldens(graph_steps, manifest):
    """Nonuniform grids (their own persistent kernel), microphones (omni and
    directional rows sampled after each batch step), and members that step
    through their own plans inside the run (Mur ABC and radiation-impedance
    planes, membrane sources, a nonuniform grid with ADE materials), mixed
    with plain and ADE members: every member equals its reference fixture --
    fields, probe traces and microphone waveforms."""
    solvers = [C.build_case(API, _case(k, n)) for k, n in WIDE_MIX]
    steps = [_case(k, n)["steps"] for k, n in WIDE_MIX]
    alone = [BatchedSolver.steps_alone(s) for s in solvers]
    assert alone == [False, False, False, False, False, True, True, True, True, False, False]
    b = BatchedSolver(solvers, rows=8, i_chunk=5)
    b.run_steps(steps, graph_steps=graph_steps)
    for s, (kind, name) in zip(solvers, WIDE_MIX):
        key = ("ade_" if kind == "ade" else "plain_") + name
        info, g = manifest[key], golden(key)
        for f in ("p", "vx", "vy", "vz"):
            assert sha256(getattr(s, f)) == info[f"sha_{f}"], f"{key} {f}"
        for pn in g["probe_names"]:
            np.testing.assert_array_equal(s.get_probe_data()[str(pn)], g[f"trace__{pn}"],
                                          err_msg=f"{key} probe {pn}")
        for k in g.files:
            if k.startswith("mic__"):
                np.testing.assert_array_equal(s.microphones[k[5:]].get_waveform(), g[k],
                                              err_msg=f"{key} microphone {k[5:]}")


@pytest.mark.parametrize("graph_steps", [0, 16])
def test_batch_matches_reference_goldens(graph_steps, manifest):
    """The mix (plain, solids, plane sources, Debye and Lorentz ADE, different
    step counts) in one batch reproduces each case's reference fixture."""
    solvers = [C.build_case(API, _case(k, n)) for k, n in MIX]
    steps = [_case(k, n)["steps"] for k, n in MIX]
    b = BatchedSolver(solvers, rows=8, i_chunk=5)
    b.run_steps(steps, graph_steps=graph_steps)
    for s, (kind, name) in zip(solvers, MIX):
        key = ("ade_" if kind == "ade" else "plain_") + name
        info, g = manifest[key], golden(key)
        for f in ("p", "vx", "vy", "vz"):
            assert sha256(getattr(s, f)) == info[f"sha_{f}"], f"{key} {f}"
        for pn in g["probe_names"]:
            np.testing.assert_array_equal(s.get_probe_data()[str(pn)], g[f"trace__{pn}"])
        if kind == "ade" and s._ade_debye:
            np.testing.assert_array_equal(s._ade_J_debye, g["ade_ade_J_debye"])


@pytest.mark.parametrize("kernel", ["column", "warp", "warp_prefetch", "warp_prefetch_m8"])
@pytest.mark.parametrize("rows,i_chunk", [(4, 8), (16, 32), (8, 0), (8, 3)])
def test_batch_equals_alone_in_two_runs(rows, i_chunk, kernel):
    """Members run in two batched runs (continuing state) equal the solves run
    alone with the default kernel."""
    alone = [C.build_case(API, _case(k, n)) for k, n in MIX]
    mixed = [C.build_case(API, _case(k, n)) for k, n in MIX]
    first = [17 + 3 * q for q in range(len(MIX))]
    second = [40 - 2 * q for q in range(len(MIX))]
    for s, a, b_ in zip(alone, first, second):
        s.run_steps(a)
        s.run_steps(b_)
    b = BatchedSolver(mixed, rows=rows, i_chunk=i_chunk, kernel=kernel)
    b.run_steps(first, graph_steps=8)
    b.run_steps(second, graph_steps=0)
    for s, t in zip(mixed, alone):
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(s, f), getattr(t, f))
        for name, tr in t.get_probe_data().items():
            np.testing.assert_array_equal(s.get_probe_data()[name], tr)
        assert s.step_count == t.step_count and s.time == t.time


def test_batch_autotune_leaves_state_unchanged():
    a = [C.build_case(API, _case(k, n)) for k, n in MIX]
    b = [C.build_case(API, _case(k, n)) for k, n in MIX]
    BatchedSolver(a).run_steps(20)
    BatchedSolver(b).run_steps(20)
    bs = BatchedSolver(a)
    table = bs.autotune(launches=2)
    assert table["best"][0] in S.batch.PLAIN_KERNELS
    assert table["best"][1] in (4, 8, 16)
    bs.run_steps(30)
    BatchedSolver(b).run_steps(30)
    for x, y in zip(a, b):
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(x, f), getattr(y, f))


def test_generated_batch_workload_members_equal_alone():
    """Three solves from the batch generator (64-256 edges, solids, Debye
    material, 500-3000 steps truncated to 120 here)."""
    mixed, steps, info = batch_workload(seed=3, n_solves=3)
    alone, _, _ = batch_workload(seed=3, n_solves=3)
    n = [min(120, q) for q in steps]
    BatchedSolver(mixed).run_steps(n, graph_steps=20)
    for s, q in zip(alone, n):
        s.run_steps(q)
    for x, y in zip(mixed, alone):
        for f in ("p", "vx"):
            np.testing.assert_array_equal(getattr(x, f), getattr(y, f))
        assert np.abs(x.p).max() > 0


def test_padded_twins_equal_unpadded_batch_and_follow_table_changes(manifest):
    """Members with nz % 4 != 0 run as padded twins (float4 tiles): fields,
    traces and ADE fields equal the unpadded batch's and the reference's,
    over several runs, and a probe added between runs rebuilds the twin."""
    mix = [("plain", "blocks_odd"), ("ade", "lorentz_mixed_geom"), ("plain", "plane_yz_geom")]
    assert any(_case(k, n)["shape"][2] % 4 for k, n in mix)
    a = [C.build_case(API, _case(k, n)) for k, n in mix]
    b = [C.build_case(API, _case(k, n)) for k, n in mix]
    pa = BatchedSolver(a, kernel="warp_prefetch", pad=True)
    pa.PAD_MIN_CELLS = 0  # pad this small batch too
    pb = BatchedSolver(b, kernel="warp_prefetch", pad=False)
    steps = [_case(k, n)["steps"] for k, n in mix]
    first = [n // 3 for n in steps]
    pa.run_steps(first, graph_steps=8)
    pb.run_steps(first, graph_steps=8)
    assert any(getattr(s, "_pad_twin", None) is not None for s in a)
    twins = [getattr(s, "_pad_twin", None) for s in a]
    for s in a + b:
        s.add_probe("late", tuple(n // 2 for n in s.shape))
    rest = [n - f for n, f in zip(steps, first)]
    pa.run_steps(rest, graph_steps=0)
    pb.run_steps(rest, graph_steps=0)
    for s, t in zip(a, twins):
        if t is not None:
            assert s._pad_twin is not t  # rebuilt after the table change
    for sa, sb, (kind, name) in zip(a, b, mix):
        key = ("ade_" if kind == "ade" else "plain_") + name
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(sa, f), getattr(sb, f), err_msg=f"{name} {f}")
            assert sha256(getattr(sa, f)) == manifest[key][f"sha_{f}"], f"{key} {f}"
        for pn, tr in sb.get_probe_data().items():
            np.testing.assert_array_equal(sa.get_probe_data()[pn], tr, err_msg=f"{name} {pn}")
        if kind == "ade":
            np.testing.assert_array_equal(sa._ade_J_debye, sb._ade_J_debye)
            np.testing.assert_array_equal(sa._ade_J_lorentz, sb._ade_J_lorentz)
