"""GPU parity: the sm_103a kernels against the reference's golden vectors and
the CPU oracle, bit for bit.

Tolerance: none -- FP32 fields, probe traces and masks must be identical
(the reference native path is deterministic FP32 without FMA, and so are the
kernels).  Every case goes through the public drop-in API
(strata_fdtd_gb300.FDTDSolver), i.e. through the C ABI.
"""
import types

import numpy as np
import pytest

import cases as C
from conftest import golden, sha256

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import strata_fdtd_gb300 as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

API = types.SimpleNamespace(
    FDTDSolver=S.FDTDSolver, UniformGrid=S.UniformGrid, PML=S.PML, GaussianPulse=S.GaussianPulse,
    Box=S.Box, Sphere=S.Sphere, Cylinder=S.Cylinder, Union=S.Union, Intersection=S.Intersection,
    Difference=S.Difference, HelmholtzResonator=S.HelmholtzResonator, Pole=S.Pole,
    Cone=S.Cone, Horn=S.Horn, SpiralHorn=S.SpiralHorn, HelicalTube=S.HelicalTube,
    SmoothUnion=S.SmoothUnion, SmoothIntersection=S.SmoothIntersection,
    SmoothDifference=S.SmoothDifference, LoudspeakerEnclosure=S.LoudspeakerEnclosure,
    bookshelf_speaker=S.bookshelf_speaker, tower_speaker=S.tower_speaker,
    PoleType=S.PoleType, SimpleMaterial=S.SimpleMaterial, NonuniformGrid=S.NonuniformGrid,
    MaterializedGeometry=S.MaterializedGeometry,
    ABCFirstOrder=S.ABCFirstOrder, RadiationImpedance=S.RadiationImpedance,
    CircularMembraneSource=S.CircularMembraneSource,
    RectangularMembraneSource=S.RectangularMembraneSource)
ORACLE = O.make_api()
SMALL = [k for k, v in C.PLAIN_CASES.items() if not v.get("big") and k != "c1_full"]
TILE_CONFIGS = [c for c in S.solver.kernel_configs() if c.startswith("tile")]


def _compare(solver, key, manifest, fields=True):
    info = manifest[key]
    g = golden(key)
    for name in g["probe_names"]:
        np.testing.assert_array_equal(solver.get_probe_data()[str(name)], g[f"trace__{name}"],
                                      err_msg=f"{key}: probe {name}")
    for k in g.files:
        if k.startswith("mic__"):
            np.testing.assert_array_equal(solver.microphones[k[5:]].get_waveform(), g[k],
                                          err_msg=f"{key}: microphone {k[5:]}")
    if fields:
        for f in ("p", "vx", "vy", "vz"):
            arr = getattr(solver, f)
            if f"field__{f}" in g.files:
                np.testing.assert_array_equal(arr, g[f"field__{f}"], err_msg=f"{key}: {f}")
            assert sha256(arr) == info[f"sha_{f}"], f"{key}: {f} differs from the reference"


@pytest.mark.parametrize("name", SMALL)
def test_plain_cases_one_call(name, manifest):
    case = C.PLAIN_CASES[name]
    s = C.build_case(API, case)
    s.run_steps(case["steps"])
    _compare(s, "plain_" + name, manifest)
    if case.get("geometry"):
        assert sha256(s.geometry) == manifest["plain_" + name]["sha_geometry"]


@pytest.mark.parametrize("name", ["c1_tiny", "blocks_odd", "plane_yz_geom", "mics_directional"])
def test_plain_cases_step_by_step(name, manifest):
    case = C.PLAIN_CASES[name]
    s = C.build_case(API, case)
    for q in range(case["steps"]):
        s.step()
        if q == case["steps"] // 2:
            _ = s.p[0, 0, 0]  # host read in the middle: forces a download + re-upload
    _compare(s, "plain_" + name, manifest)


@pytest.mark.parametrize("name", list(C.ADE_CASES))
def test_ade_cases(name, manifest):
    case = C.ADE_CASES[name]
    s = C.build_case(API, case)
    s.run_steps(case["steps"])
    _compare(s, "ade_" + name, manifest)
    g = golden("ade_" + name)
    np.testing.assert_array_equal(s._material_id, g["material_id"])
    if s._ade_debye:
        np.testing.assert_array_equal(s._ade_J_debye, g["ade_ade_J_debye"])
    if s._ade_lorentz:
        np.testing.assert_array_equal(s._ade_J_lorentz, g["ade_ade_J_lorentz"])
        np.testing.assert_array_equal(s._ade_J_lorentz_prev, g["ade_ade_J_lorentz_prev"])


def _check_ade(s, name, manifest):
    _compare(s, "ade_" + name, manifest)
    g = golden("ade_" + name)
    if s._ade_debye:
        np.testing.assert_array_equal(s._ade_J_debye, g["ade_ade_J_debye"])
    if s._ade_lorentz:
        np.testing.assert_array_equal(s._ade_J_lorentz, g["ade_ade_J_lorentz"])
        np.testing.assert_array_equal(s._ade_J_lorentz_prev, g["ade_ade_J_lorentz_prev"])


@pytest.mark.parametrize("config", ["cell"] + [c for c in S.solver.kernel_configs()
                                               if c.startswith("tile")])
@pytest.mark.parametrize("name", ["split_boxes_geom", "lorentz_mixed_geom", "nu_mixed_geom",
                                  "materialized_sdf"])
def test_ade_split_step_every_tile_config(name, config, manifest):
    """ADE steps split between a warp-tile kernel (outside the material
    boxes, rounded out to its tiles) and the per-cell ADE kernel (inside):
    fields, traces and J equal the reference's for every configuration."""
    case = C.ADE_CASES[name]
    s = C.build_case(API, case)
    s.set_kernel(config, 3 if config.startswith("tile1") else 0)
    s.run_steps(case["steps"] // 2)
    s.run_steps(case["steps"] - case["steps"] // 2)
    _check_ade(s, name, manifest)


def test_materialized_geometry_voxelised_in_one_pass():
    """voxelize_with_materials on the GPU (one kernel for the geometry and
    every region) equals the reference's mask and ids, on the uniform grid of
    the golden case and on a stretched grid against the oracle's NumPy
    restatement; MaterialVolume regions behave as Box regions."""
    case = C.ADE_CASES["materialized_sdf"]
    g = golden("ade_materialized_sdf")
    geo = S.MaterializedGeometry(C.sdf_tree(API, "mat_air"))
    ref = O.MaterializedGeometry(C.sdf_tree(ORACLE, "mat_air"))
    for which, m in case["materialized"]["regions"]:
        geo.set_material(C.sdf_tree(API, which), C._material(API, m))
        ref.set_material(C.sdf_tree(ORACLE, which), None)
    grid = S.UniformGrid(case["shape"], case["res"])
    mask, ids = geo.voxelize_with_materials(grid)
    np.testing.assert_array_equal(mask, np.unpackbits(g["geometry"])[: mask.size].reshape(
        mask.shape).astype(bool))
    np.testing.assert_array_equal(ids, g["material_id"])
    assert geo.material_count() == 4 and set(geo.get_material_table()) == {0, 1, 2, 3}
    nu = S.NonuniformGrid.from_stretch((40, 36, 44), 1e-3, 1.02, 1.0, 1.03, center_fine=True)
    onu = O.NonuniformGrid.from_stretch((40, 36, 44), 1e-3, 1.02, 1.0, 1.03, center_fine=True)
    mask2, ids2 = geo.voxelize_with_materials(nu)
    rmask, rids = ref.voxelize_with_materials(onu)
    np.testing.assert_array_equal(mask2, rmask)
    np.testing.assert_array_equal(ids2, rids)
    vol = S.MaterialVolume.from_corners((0.0, 0.0, 0.03), (0.013, 0.036, 0.044), None)
    geo2 = S.MaterializedGeometry(C.sdf_tree(API, "mat_air"))
    geo2.set_material(vol.region, C._material(API, case["materialized"]["regions"][2][1]))
    _, ids3 = geo2.voxelize_with_materials(grid)
    slab = C.sdf_tree(API, "mat_slab").voxelize(grid) & mask
    np.testing.assert_array_equal(ids3, slab.astype(np.uint8))


def test_ade_autotune_then_steps(manifest):
    case = C.ADE_CASES["split_boxes_geom"]
    s = C.build_case(API, case)
    s.run_steps(10)
    table = s.autotune(launches=2)
    assert table["best"].startswith("tile")
    s.run_steps(case["steps"] - 10)
    _check_ade(s, "split_boxes_geom", manifest)


@pytest.mark.parametrize("config", TILE_CONFIGS + ["auto", "col1", "cell"])
@pytest.mark.parametrize("name", ["nu_stretch_blocks", "nu_regions_sdf"])
def test_nonuniform_every_config(name, config, manifest):
    """Nonuniform grids run the warp-tile kernels with per-face coefficients
    and per-cell divergence scales; a configuration without them falls back
    to the default warp tiles.  Fields and traces equal the reference's
    update_velocity/pressure_nonuniform path."""
    case = C.PLAIN_CASES[name]
    s = C.build_case(API, case)
    s.set_kernel(config, 3 if config.startswith("tile1") else 0)
    s.run_steps(case["steps"] // 3)
    s.run_steps(case["steps"] - case["steps"] // 3)
    _compare(s, "plain_" + name, manifest)


@pytest.mark.parametrize("config", ["tile_r1_w4", "tile1_r2_w8", "col4", "cell"])
@pytest.mark.parametrize("name", ["abc_all_sources", "rad_pml_mix"])
def test_plane_boundaries(name, config, manifest):
    """Mur ABC and radiation-impedance planes after the fused step, sources
    after them, stored planes carried across calls; reset() clears them."""
    case = C.PLAIN_CASES[name]
    s = C.build_case(API, case)
    s.set_kernel(config)
    s.run_steps(25)
    s.reset()
    for _ in range(5):
        s.step()
    s.run_steps(case["steps"] - 5)
    _compare(s, "plain_" + name, manifest)
    with pytest.raises(NotImplementedError):
        s.add_boundary(S.PML(depth=2))  # a PML after plane boundaries
    assert S.BatchedSolver.steps_alone(s)  # a batch steps it through its own plan


def test_membranes_step_by_step_and_limits(manifest):
    """Membrane sources injected after the fused step (velocity injection
    included), step by step with a host read in the middle."""
    case = C.PLAIN_CASES["membranes"]
    s = C.build_case(API, case)
    for q in range(case["steps"]):
        s.step()
        if q == 37:
            _ = s.vx[0, 0, 0]
    _compare(s, "plain_membranes", manifest)
    assert S.BatchedSolver.steps_alone(C.build_case(API, case))


def test_nonuniform_autotune_and_limits(manifest):
    case = C.PLAIN_CASES["nu_stretch_low_end"]
    s = C.build_case(API, case)
    s.run_steps(7)
    table = s.autotune(launches=2)
    assert table["best"].startswith("tile")
    s.run_steps(case["steps"] - 7)
    _compare(s, "plain_nu_stretch_low_end", manifest)
    assert not S.BatchedSolver.steps_alone(s)  # batched: its own persistent kernel


def test_c1_quick_start_1000_steps(manifest):
    """The reference quick start, 100^3 x 1000 steps, through run(duration)."""
    case = C.PLAIN_CASES["c1_full"]
    s = C.build_case(API, case)
    s.run(duration=case["steps"] * s.dt * 0.9999)
    assert s.step_count == 1000
    _compare(s, "plain_c1_full", manifest)


def test_c2_enclosure_full_size_20_steps(manifest):
    """400^3 with the GPU-voxelised enclosure: mask, traces and fields equal
    the reference's after 20 steps."""
    case = C.PLAIN_CASES["c2_enclosure_20"]
    info = manifest["plain_c2_enclosure_20"]
    s = S.FDTDSolver(grid=S.UniformGrid(case["shape"], case["res"]), c=343.0, rho=1.204,
                     courant=0.5, backend="native")
    s.add_boundary(S.PML(depth=16))
    s.set_geometry_sdf(C.c2_solid(API))
    assert sha256(s.geometry) == info["sha_geometry"]
    s.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0, amplitude=1.0))
    for name, pos in info["probes"]:
        s.add_probe(name, tuple(pos))
    s.run_steps(case["steps"])
    _compare(s, "plain_c2_enclosure_20", manifest)


@pytest.mark.parametrize("name", list(C.VOXEL_CASES))
def test_voxelize_matches_reference(name):
    shape, res, which = C.VOXEL_CASES[name]
    grid = S.UniformGrid(shape, res)
    mask = C.sdf_tree(API, which).voxelize(grid)
    ref = np.unpackbits(golden("voxel")["mask__" + name])[: mask.size].reshape(shape).astype(bool)
    if which in C.VOXEL_ROUNDING_CASES:
        # np.dot / matmul round through BLAS; only cells within rounding of a surface may differ
        diff = mask != ref
        if diff.any():
            # the oracle's distances (the builder's own for the loudspeaker
            # cabinet, which the oracle does not restate)
            checker = API if which in ("bookshelf", "cabinet") else ORACLE
            d = C.sdf_tree(checker, which).sdf(np.stack(np.meshgrid(
                grid.x_coords, grid.y_coords, grid.z_coords, indexing="ij"), -1).reshape(-1, 3))
            assert np.all(np.abs(d.reshape(shape)[diff]) < 1e-15)
    else:
        np.testing.assert_array_equal(mask, ref)


def test_sdf_point_evaluation_matches_oracle():
    tree = C.sdf_tree(API, "csg_mix")
    pts = np.random.default_rng(0).uniform(0, 0.05, (5000, 3))
    np.testing.assert_array_equal(tree.sdf(pts), C.sdf_tree(ORACLE, "csg_mix").sdf(pts))


def _random_case(seed):
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(5, 41, size=3))
    pml = int(rng.integers(1, max(2, min(shape) // 3)))
    axes = [("x", "y", "z"), ("x",), ("y", "z"), ("z",)][int(rng.integers(0, 4))]
    srcs = []
    for _ in range(int(rng.integers(1, 4))):
        if rng.random() < 0.7:
            srcs.append(("point", tuple(int(rng.integers(0, n)) for n in shape),
                         float(rng.uniform(5e3, 4e4)), float(rng.uniform(-2, 2))))
        else:
            ax = int(rng.integers(0, 3))
            srcs.append(("plane", {"axis": ax, "index": int(rng.integers(0, shape[ax]))},
                         float(rng.uniform(5e3, 4e4)), 1.0))
    probes = [(f"q{q}", tuple(int(rng.integers(0, n)) for n in shape)) for q in range(3)]
    case = dict(shape=shape, res=float(rng.choice([1e-3, 2e-3, 5e-4])),
                courant=float(rng.uniform(0.3, 0.99)), pml=dict(depth=pml, axis=axes),
                sources=srcs, probes=probes, steps=int(rng.integers(20, 90)))
    if rng.random() < 0.7:
        case["geometry"] = dict(kind="blocks", seed=int(seed), n_boxes=2, n_spheres=1)
    return case


@pytest.mark.parametrize("seed", range(12))
def test_random_cases_against_oracle(seed):
    case = _random_case(seed)
    try:
        ref = C.build_case(ORACLE, case)
    except (IndexError, ValueError):
        pytest.skip("case outside what the reference accepts")
    ref.run_steps(case["steps"])
    s = C.build_case(API, case)
    s.run_steps(case["steps"])
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"seed {seed} {f}")
    for name in ref.get_probe_data():
        np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name])


@pytest.mark.parametrize("variant,i_chunk", [("cell", 0), ("march", 1), ("march", 3), ("col", 0),
                                             ("col", 1), ("col", 5), ("col1", 0), ("col1", 2),
                                             ("march", 7), ("march", 0)])
@pytest.mark.parametrize("seed", [0, 3, 5, 8])
def test_kernel_variants_against_oracle(seed, variant, i_chunk):
    case = _random_case(100 + seed)
    try:
        ref = C.build_case(ORACLE, case)
    except (IndexError, ValueError):
        pytest.skip("case outside what the reference accepts")
    ref.run_steps(case["steps"])
    s = C.build_case(API, case)
    s.set_kernel(variant, i_chunk)
    s.run_steps(case["steps"])
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"{variant} {f}")
    for name in ref.get_probe_data():
        np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name])


@pytest.mark.parametrize("shape,ich", [((9, 7, 8), 0), ((17, 21, 36), 0), ((12, 30, 132), 5),
                                       ((40, 9, 8), 1), ((33, 40, 40), 0)])
def test_col_float4_against_oracle(shape, ich):
    """The float4 column kernel (nz % 4 == 0) with solids, a plane source
    along k and sources on the float4 lane boundaries."""
    case = dict(shape=shape, res=1e-3, courant=0.6, pml=dict(depth=2),
                geometry=dict(kind="blocks", seed=sum(shape), n_boxes=2, n_spheres=1),
                sources=[("point", (shape[0] // 2, shape[1] // 2, 3), 25000.0, 1.0),
                         ("plane", {"axis": 2, "index": shape[2] - 1}, 15000.0, 0.7),
                         ("point", (1, 1, 0), 30000.0, -1.0)],
                probes=[("a", (shape[0] // 2, shape[1] // 2, shape[2] // 2)),
                        ("b", (shape[0] - 1, shape[1] - 1, shape[2] - 1))], steps=70)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(case["steps"])
    s = C.build_case(API, case)
    s.set_kernel("col", ich)
    s.run_steps(case["steps"])
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"{shape} {f}")
    for name in ref.get_probe_data():
        np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name])


@pytest.mark.parametrize("config", S.solver.kernel_configs()[1:])
def test_every_kernel_config_against_oracle(config):
    """Each column-kernel configuration (vector width, rows, register cap,
    streaming stores) on a float4-compatible grid and an odd one."""
    for shape in ((20, 18, 36), (15, 13, 22)):
        case = dict(shape=shape, res=1e-3, courant=0.55, pml=dict(depth=3),
                    geometry=dict(kind="blocks", seed=shape[2], n_boxes=2, n_spheres=1),
                    sources=[("point", (5, 6, 7), 25000.0, 1.0),
                             ("plane", {"axis": 1, "index": 2}, 12000.0, 0.3)],
                    probes=[("a", (10, 9, 11))], steps=45)
        ref = C.build_case(ORACLE, case)
        ref.run_steps(case["steps"])
        s = C.build_case(API, case)
        s.set_kernel(config, 3 if shape[0] == 15 else 0)
        s.run_steps(case["steps"])
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"{config} {f}")
        np.testing.assert_array_equal(s.get_probe_data()["a"], ref.get_probe_data()["a"])


@pytest.mark.parametrize("config", TILE_CONFIGS)
@pytest.mark.parametrize("shape,ich", [((19, 37, 36), 0), ((12, 21, 132), 5), ((9, 5, 64), 1),
                                       ((7, 1, 8), 0), ((6, 3, 4), 2), ((25, 70, 44), 4),
                                       ((10, 17, 20), 0), ((8, 33, 28), 3)])
def test_warp_tile_kernels_against_oracle(config, shape, ich):
    """The warp-tile kernels (lane-shuffled neighbours): rows across lane
    groups and warps, k across lanes and tiles, partial tiles in j and k, every
    source kind on lane and group boundaries, two sources on one cell."""
    nx, ny, nz = shape
    sources = [("point", (nx // 2, min(ny - 1, 4), min(nz - 1, 3)), 25000.0, 1.0),
               ("point", (nx // 2, min(ny - 1, 4), min(nz - 1, 3)), 17000.0, -0.4),
               ("point", (1, min(ny - 1, 3), min(nz - 1, 4)), 30000.0, 0.8),
               ("point", (nx - 2, ny - 1, nz - 1), 21000.0, 0.5),
               ("plane", {"axis": 0, "index": nx // 3}, 9000.0, 0.2),
               ("plane", {"axis": 1, "index": min(ny - 1, 8)}, 12000.0, 0.3),
               ("plane", {"axis": 2, "index": min(nz - 1, 32)}, 15000.0, 0.25)]
    axes = tuple(ax for ax, n in zip("xyz", shape) if n >= 6)
    case = dict(shape=shape, res=1e-3, courant=0.6, pml=dict(depth=2, axis=axes),
                sources=sources,
                probes=[("a", (nx // 2, ny // 2, nz // 2)), ("b", (nx - 1, ny - 1, nz - 1))],
                steps=50)
    for geometry in ((True, False) if min(shape) >= 8 else (False,)):
        if geometry:
            case = dict(case, geometry=dict(kind="blocks", seed=sum(shape), n_boxes=2, n_spheres=1))
        else:
            case = {k: v for k, v in case.items() if k != "geometry"}
        ref = C.build_case(ORACLE, case)
        ref.run_steps(case["steps"])
        s = C.build_case(API, case)
        s.set_kernel(config, ich)
        s.run_steps(case["steps"])
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(s, f), getattr(ref, f),
                                          err_msg=f"{config} {shape} geometry={geometry} {f}")
        for name in ref.get_probe_data():
            np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name])


def test_autotune_leaves_state_unchanged():
    case = C.PLAIN_CASES["blocks_odd"]
    a = C.build_case(API, case)
    b = C.build_case(API, case)
    a.run_steps(50)
    b.run_steps(50)
    table = a.autotune(launches=3)
    assert table["best"] in S.solver.kernel_configs()
    assert all(v > 0 for k, v in table.items() if k != "best")
    a.run_steps(40)
    b.run_steps(40)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))


@pytest.mark.parametrize("variant", ["cell", "march", "col", "col1"])
def test_c1_quick_start_both_kernels(variant, manifest):
    case = C.PLAIN_CASES["c1_full"]
    s = C.build_case(API, case)
    s.set_kernel(variant)
    s.run_steps(case["steps"])
    _compare(s, "plain_c1_full", manifest)


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 6, 9), (7, 1, 5), (4, 5, 1), (2, 2, 2)])
def test_degenerate_shapes_against_oracle(shape):
    case = dict(shape=shape, res=1e-3, courant=0.5, pml=None, impulse=((0, 0, 0), 1.0),
                sources=[("point", (0, 0, 0), 20000.0, 1.0)], probes=[("a", (0, 0, 0))],
                steps=25)
    ref = C.build_case(ORACLE, case)
    ref.run_steps(25)
    s = C.build_case(API, case)
    s.run_steps(25)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f))


def test_full_size_against_oracle_and_scaling_property():
    """400^3 with the enclosure: 6 steps bit-exact against the C oracle, and
    doubling the source amplitude doubles every field exactly (FP32 scaling
    by 2 commutes with every rounding) over 60 steps."""
    solid = C.c2_solid(API)
    a = S.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    a.add_boundary(S.PML(depth=16))
    a.set_geometry_sdf(solid)
    a.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0, amplitude=1.0))
    a.add_probe("x", (200, 200, 230))
    o = O.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    o.add_boundary(O.PML(depth=16))
    o.set_geometry(a.geometry)
    o.add_source(O.GaussianPulse(position=(200, 200, 200), frequency=2000.0, amplitude=1.0))
    # a nonzero state so the stencil is exercised everywhere
    rng = np.random.default_rng(7)
    init = rng.standard_normal((400, 400, 400), dtype=np.float32) * np.float32(1e-3)
    init[~a.geometry] = 0.0
    a.p = init.copy()
    o.p = init
    a.run_steps(6)
    o.run_steps(6)
    for f in ("p", "vx", "vy", "vz"):
        assert sha256(getattr(a, f)) == sha256(getattr(o, f)), f
    b = S.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    b.add_boundary(S.PML(depth=16))
    b.set_geometry_sdf(solid)
    b.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0, amplitude=2.0))
    c1 = S.FDTDSolver(shape=(400, 400, 400), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
    c1.add_boundary(S.PML(depth=16))
    c1.set_geometry_sdf(solid)
    c1.add_source(S.GaussianPulse(position=(200, 200, 200), frequency=2000.0, amplitude=1.0))
    b.run_steps(60)
    c1.run_steps(60)
    for f in ("p", "vx"):
        x1, x2 = getattr(c1, f), getattr(b, f)
        assert np.abs(x1).max() > 0
        # exact where the values are normal; subnormal results round on an
        # absolute grid, so scaling is not exact there
        normal = np.abs(x1) > 1e-30
        assert normal.sum() > 1000
        np.testing.assert_array_equal(x2[normal], 2 * x1[normal])
        np.testing.assert_allclose(x2[~normal], 2 * x1[~normal], rtol=0, atol=1e-37)


def test_host_edits_between_steps_are_seen():
    """solver.p[...] = v between steps, as the reference tests do
    (tests/test_native_extension.py:247-249)."""
    case = dict(shape=(20, 22, 24), res=1e-3, courant=0.5, pml=dict(depth=3), sources=[],
                probes=[("c", (10, 11, 12))], steps=30)
    s = C.build_case(API, case)
    o = C.build_case(ORACLE, case)
    for solver in (s, o):
        solver.p[10, 11, 12] = 1.0
        for q in range(30):
            solver.step()
            if q == 10:
                solver.vx[3, 4, 5] = 0.25
    np.testing.assert_array_equal(s.p, o.p)
    np.testing.assert_array_equal(s.get_probe_data()["c"], o.get_probe_data()["c"])


def test_energy_matches_host_sum():
    case = C.PLAIN_CASES["blocks_odd"]
    s = C.build_case(API, case)
    s.run_steps(80)
    e = s.compute_energy()
    g = s.geometry
    dV = s.dx**3
    pe = 0.5 * np.sum(s.p[g].astype(np.float64) ** 2) / (s.rho * s.c**2) * dV
    v2 = s.vx.astype(np.float64) ** 2 + s.vy.astype(np.float64) ** 2 + s.vz.astype(np.float64) ** 2
    ke = 0.5 * s.rho * np.sum(v2[g]) * dV
    assert e == pytest.approx(pe + ke, rel=1e-12)


def test_errors_are_loud():
    with pytest.raises(ValueError):
        S.FDTDSolver(shape=(8, 8, 8), resolution=1e-3, backend="python")
    s = S.FDTDSolver(shape=(8, 8, 8), resolution=1e-3)
    with pytest.raises(ValueError):
        s.add_source(S.GaussianPulse(position=(9, 0, 0), frequency=1000.0))
    with pytest.raises(ValueError):
        s.add_microphone(position=(0.001, 0.001, 0.001), name="card", pattern="cardioid5")
    with pytest.raises(ValueError):
        s.add_microphone(position=(0.001, 0.001, 0.001), name="par", pattern="figure8",
                         direction=(0, 0, 2))
    with pytest.raises(ValueError):
        s.add_microphone(position=(0.0079, 0.001, 0.001), name="outside")


def test_padded_twin_and_its_fallback_against_oracle():
    """nz % 4 != 0 with the automatic kernel: long runs step through the
    padded twin (float4 tiles).  A nonzero last vz plane (which the
    reference never updates and the twin would hold at zero) set before the
    first run, or edited between runs, sends the solve back to its own plan;
    every variant equals the oracle bit for bit."""
    case = dict(shape=(21, 26, 31), res=1e-3, courant=0.55, pml=dict(depth=3),
                geometry=dict(kind="blocks", seed=4, n_boxes=2, n_spheres=1),
                sources=[("point", (10, 12, 14), 25000.0, 1.0),
                         ("plane", {"axis": 0, "index": 5}, 9000.0, 0.2)],
                probes=[("a", (10, 13, 30)), ("b", (4, 4, 4))], steps=80)
    rng = np.random.default_rng(3)
    edge = np.zeros((21, 26), np.float32)
    edge[::3, ::2] = rng.standard_normal(edge[::3, ::2].shape).astype(np.float32) * 1e-3
    for when in ("none", "before", "between"):
        ref = C.build_case(ORACLE, case)
        s = C.build_case(API, case)
        if when == "before":
            ref.vz[:, :, -1] = edge
            s.vz[:, :, -1] = edge
        ref.run_steps(40)
        s.run_steps(40)
        assert (getattr(s, "_pad_twin", None) is not None) == (when != "before"), when
        if when == "between":
            ref.vz[:, :, -1] = edge
            vz = s.vz
            vz[:, :, -1] = edge
        ref.run_steps(40)
        s.run_steps(40)
        if when == "between":  # the edit was seen: the second run used the solve's own plan
            assert s._pad_twin is None
        # ("before": the PML decays the set plane to exactly zero within the
        # first run, after which the twin is valid again)
        for f in ("p", "vx", "vy", "vz"):
            np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f"{when} {f}")
        for name in ref.get_probe_data():
            np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name])


def test_graph_replays_follow_table_changes_against_oracle():
    """Runs of 50 steps or more replay captured CUDA graphs: a probe added
    between runs, a host edit of p, runs that leave remainders, a kernel
    chosen and then automatic again; fields and every probe trace equal the
    oracle's, and the graph cache is rebuilt after each table change."""
    case = dict(shape=(30, 33, 40), res=1e-3, courant=0.5, pml=dict(depth=4),
                geometry=dict(kind="blocks", seed=9, n_boxes=2, n_spheres=1),
                sources=[("point", (15, 16, 20), 20000.0, 1.0),
                         ("plane", {"axis": 2, "index": 6}, 11000.0, 0.2)],
                probes=[("a", (10, 11, 12))], steps=0)
    ref = C.build_case(ORACLE, case)
    s = C.build_case(API, case)
    for x in (ref, s):
        x.run_steps(120)
    stamp = s._graphs["stamp"]
    for x in (ref, s):
        x.add_probe("b", (25, 20, 30))
        x.run_steps(75)
    assert s._graphs["stamp"] != stamp
    ref.p[5, 6, 7] += np.float32(0.25)
    p = s.p
    p[5, 6, 7] += np.float32(0.25)
    for x in (ref, s):
        x.run_steps(100)
    s.set_kernel("tile1_r2_w4")
    ref.run_steps(60)
    s.run_steps(60)
    s.set_kernel("auto")
    ref.run_steps(150)
    s.run_steps(150)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(s, f), getattr(ref, f), err_msg=f)
    for name in ref.get_probe_data():
        np.testing.assert_array_equal(s.get_probe_data()[name], ref.get_probe_data()[name],
                                      err_msg=name)


@pytest.mark.parametrize("which", ["cone_smooth", "horns", "horn_oblique", "spiral_horn",
                                   "helical_tube"])
def test_curved_shapes_point_evaluation_matches_oracle(which):
    """Cones, horns, the smooth blends and the path-swept shapes evaluated at
    random points on the GPU against the oracle's NumPy restatement, within
    the rounding of BLAS dot products and transcendental functions."""
    pts = np.random.default_rng(7).uniform(-0.005, 0.065, (3000, 3))
    got = C.sdf_tree(API, which).sdf(pts)
    want = C.sdf_tree(ORACLE, which).sdf(pts)
    assert np.all(np.isfinite(want))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-15)


def test_audio_file_waveform_drives_a_membrane_like_the_oracle(tmp_path):
    """An audio file (int16 WAV at 48 kHz, resampled to the step rate) as the
    waveform of a circular membrane: fields and traces equal the oracle's
    run with the same waveform object, bit for bit."""
    from scipy.io import wavfile

    sr = 48000
    t = np.arange(480) / sr
    tone = (np.sin(2 * np.pi * 3000 * t) * np.hanning(t.size) * 20000).astype(np.int16)
    path = tmp_path / "tone.wav"
    wavfile.write(path, sr, tone)
    wf = S.AudioFileWaveform(str(path), amplitude=0.8)

    def build(mod):
        s = mod.FDTDSolver(shape=(30, 26, 32), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
        s.add_boundary(mod.PML(depth=4))
        s.add_source(mod.CircularMembraneSource(center=(0.015, 0.013, 0.0085), normal_axis="z",
                                                radius=0.006, mode=(0, 1), waveform=wf))
        s.add_probe("a", (15, 13, 20))
        return s

    gpu, ref = build(S), build(ORACLE)
    gpu.run_steps(90)
    ref.run_steps(90)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(gpu, f), getattr(ref, f), err_msg=f)
    np.testing.assert_array_equal(gpu.get_probe_data()["a"], ref.get_probe_data()["a"])
    assert np.abs(gpu.get_probe_data()["a"]).max() > 0


def test_library_materials_step_like_the_oracle():
    """Predefined and modelled materials (a porous JCA fit, a damping layer,
    a membrane absorber and a quarter-wave resonator: Debye and Lorentz,
    density and modulus poles) in material boxes, stepped on the GPU and by
    the oracle from the same material objects: fields and traces equal."""
    from strata_fdtd_gb300 import materials as M

    mats = [(1, M.POLYESTER_BATTING, ((6, 14), (5, 13), (8, 18))),
            (2, M.MembraneAbsorber(name="m", surface_density=4.2, cavity_depth=0.15),
             ((15, 22), (12, 20), (14, 24))),
            (3, M.QuarterWaveResonator(name="q", length=0.2, loss_factor=0.2),
             ((4, 10), (14, 20), (20, 27)))]

    def build(mod):
        s = mod.FDTDSolver(shape=(26, 24, 30), resolution=1e-3, c=343.0, rho=1.204, courant=0.5)
        s.add_boundary(mod.PML(depth=3))
        for mid, mat, box in mats:
            s.register_material(mat, material_id=mid)
            s.set_material_box(mid, *box)
        s.add_source(mod.GaussianPulse(position=(13, 12, 15), frequency=15000.0))
        s.add_probe("a", (18, 16, 20))
        s.add_probe("b", (8, 8, 10))
        return s

    gpu, ref = build(S), build(ORACLE)
    gpu.run_steps(100)
    ref.run_steps(100)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(gpu, f), getattr(ref, f), err_msg=f)
    for n in ("a", "b"):
        np.testing.assert_array_equal(gpu.get_probe_data()[n], ref.get_probe_data()[n])
    assert np.all(np.isfinite(gpu.p)) and np.abs(gpu.get_probe_data()["a"]).max() > 0


def test_tower_speaker_and_cabinet_solve():
    """The three-way tower voxelised at 4 mm has the reference's solid cell
    count; a bookshelf cabinet's mask, its woofer as a membrane source and
    an absorber region of a library material step on the GPU exactly as the
    oracle steps the same inputs."""
    from strata_fdtd_gb300 import materials as M

    g = golden("analysis_values")
    tower = S.tower_speaker(0.22, 0.3, 0.9, 0.17, 0.13, 0.025).build()
    assert int(tower.voxelize(S.UniformGrid((55, 75, 225), 4e-3)).sum()) == int(
        g["tower_inside_4mm"][0])

    enc = S.bookshelf_speaker(0.06, 0.07, 0.09, 0.03, 0.012, port_diameter=0.012,
                              port_length=0.03)
    enc._drivers[1]["waveform"] = S.GaussianPulse(position=(0, 0, 0), frequency=6000.0)
    enc.add_absorber_region(((0.01, 0.03, 0.05), (0.05, 0.06, 0.08)), material_id=1)
    grid = S.UniformGrid((40, 46, 56), 2e-3)
    air = ~enc.build().voxelize(grid)
    (box, mid), = enc.get_material_regions()
    src, = enc.get_membrane_sources()

    def build(mod):
        s = mod.FDTDSolver(shape=grid.shape, resolution=2e-3, c=343.0, rho=1.204, courant=0.5)
        s.add_boundary(mod.PML(depth=4))
        s.set_geometry(air)
        s.register_material(M.POLYESTER_BATTING, material_id=mid)
        lo = [int(round(v / 2e-3)) for v in box.center - box.size / 2]
        hi = [int(round(v / 2e-3)) for v in box.center + box.size / 2]
        s.set_material_box(mid, *zip(lo, hi))
        s.add_source(mod.CircularMembraneSource(center=src.center, radius=src.radius,
                                                normal_axis=src.normal_axis, mode=src.mode,
                                                waveform=src.waveform))
        s.add_probe("front", (20, 4, 20))
        return s

    gpu, ref = build(S), build(ORACLE)
    gpu.run_steps(80)
    ref.run_steps(80)
    for f in ("p", "vx", "vy", "vz"):
        np.testing.assert_array_equal(getattr(gpu, f), getattr(ref, f), err_msg=f)
    np.testing.assert_array_equal(gpu.get_probe_data()["front"], ref.get_probe_data()["front"])


@pytest.mark.parametrize("seed", range(12))
def test_random_sdf_trees_match_oracle(seed):
    """Seeded random trees of every shape (box, sphere, cylinder, cone, the
    four horn flares) under every operator (sharp and smooth CSG, translate,
    scale, rotate): GPU point evaluation against the oracle's NumPy
    restatement within the rounding of BLAS products and transcendental
    functions."""
    tree_g = C.random_sdf_tree(API, np.random.default_rng(seed))
    tree_o = C.random_sdf_tree(ORACLE, np.random.default_rng(seed))
    pts = np.random.default_rng(100 + seed).uniform(0.0, 0.05, (4000, 3))
    want = tree_o.sdf(pts)
    assert np.all(np.isfinite(want))
    np.testing.assert_allclose(tree_g.sdf(pts), want, rtol=0, atol=2e-15)
