"""CPU-only checks of the product: the C-ABI library loads and exports every
symbol that include/sf_gb300.h declares, and the host-side arithmetic that
feeds the kernels (coefficients, PML profiles and decays, waveform values,
pole coefficients, SDF programs) equals the reference's values stored in
tests/golden/.  No compute call is made without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import strata_fdtd_gb300 as S
from conftest import ROOT, golden
from strata_fdtd_gb300 import _native
from strata_fdtd_gb300.solver import step_coefficients


@pytest.fixture(scope="module")
def lib():
    _native.build()
    return _native.load()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sf_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(sf_\w+)\s*\(", text, re.M)))


def test_header_declares_the_abi():
    names = declared_symbols()
    for must in ("sf_plan_create", "sf_plan_step", "sf_voxelize", "sf_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(declared_symbols()) <= set(_native.SIGNATURES), "ctypes signatures incomplete"


def test_version_and_error_strings_without_gpu(lib):
    assert lib.sf_version().startswith(b"strata_fdtd_gb300")
    # argument validation happens before any device call
    assert lib.sf_plan_create(None, None) != 0
    assert b"NULL" in lib.sf_last_error()
    desc = _native.SfGridDesc(0, 4, 4, 0.0, 0.0, 0)
    plan = ctypes.c_void_p()
    assert lib.sf_plan_create(ctypes.byref(desc), ctypes.byref(plan)) != 0
    assert b"dimensions" in lib.sf_last_error()


def test_step_coefficients_match_reference(manifest):
    for key, case in (("plain_c1_full", dict(shape=(100, 100, 100), res=1e-3, c=343.0, rho=1.204,
                                             courant=0.5)),
                      ("plain_impulse_default_coeffs", dict(shape=(20, 20, 20), res=2e-3, c=343.0,
                                                            rho=1.2, courant=0.95))):
        g = S.UniformGrid(case["shape"], case["res"])
        dt, cv, cp = step_coefficients(g, case["c"], case["rho"], case["courant"])
        info = manifest[key]
        assert (dt, cv, cp) == (info["dt"], info["coeff_v"], info["coeff_p"])


def test_pml_profile_and_host_decay_match_reference():
    h = golden("host_values")
    from oracle import oracle as O
    for n, depth, res, courant in ((100, 10, 1e-3, 0.5), (37, 6, 2e-3, 0.9), (400, 16, 1e-3, 0.5)):
        pml = S.PML(depth=depth, axis="x")

        class _Stub:
            shape = (n, 4, 4)
            c = 343.0
            grid = S.UniformGrid((n, 4, 4), res)

        pml.initialize(_Stub())
        np.testing.assert_array_equal(pml.sigmas[0], h[f"sigma__{n}"])
        dt = step_coefficients(_Stub.grid, 343.0, 1.204, courant)[0]
        assert dt == h[f"dt__{n}"][0]
        # the oracle's expf restatement and the reference decays agree
        out = np.zeros(n, dtype=np.float32)
        O.lib().orc_pml_decay_f32(pml.sigmas[0].ctypes.data, n, float(np.float32(dt)),
                                  out.ctypes.data)
        np.testing.assert_array_equal(out, h[f"decay__{n}"])


def test_waveform_and_pole_coefficients_match_reference():
    h = golden("host_values")
    for f in (1000, 2000, 20000):
        g = S.GaussianPulse(position=(0, 0, 0), frequency=float(f),
                            bandwidth=15000.0 if f == 20000 else None, amplitude=1.3)
        dt = 0.5 * (1e-3 / (343.0 * np.sqrt(3)))
        vals = [g.waveform(np.array([t]), dt)[0] for t in h[f"wave_t__{f}"]]
        np.testing.assert_array_equal(np.array(vals), h[f"wave__{f}"])
    for row in h["pole_rows"]:
        dt, kind = row[0], int(row[1])
        if kind == 0:
            p = S.Pole(S.PoleType.DEBYE, delta_chi=row[3], target="density", tau=row[2])
            assert p.fdtd_coefficients(dt) == tuple(row[4:6])
        else:
            p = S.Pole(S.PoleType.LORENTZ, delta_chi=0.2, target="modulus", omega_0=row[2],
                       gamma=row[3])
            assert p.fdtd_coefficients(dt) == tuple(row[4:7])


def test_sdf_program_layout():
    tree = S.Difference(S.Box(center=(0.1, 0.1, 0.1), size=(0.2, 0.1, 0.3)),
                        S.Sphere(center=(0.1, 0.1, 0.1), radius=0.02),
                        S.Cylinder(p1=(0.1, 0.1, 0.0), p2=(0.1, 0.1, 0.05), radius=0.01)
                        .translate((0.0, 0.0, 0.001)))
    prog, n = tree.program()
    ops = [prog[q].op for q in range(n)]
    # difference folded left: max(max(box, -sphere), -translated cylinder)
    assert ops == [1, 2, 12, 20, 3, 22, 12]
    assert prog[2].n == 2 and prog[n - 1].n == 2
    assert prog[4].s0 == 0.05 and prog[4].b[2] == 1.0
    assert ctypes.sizeof(_native.SfSdfNode) == 72
    assert ctypes.sizeof(_native.SfPole) == 48


def test_helmholtz_constants_match_oracle_construction():
    from oracle import oracle as O
    for shape, size in (("box", (0.016, 0.014, 0.012)), ("sphere", (0.008,)),
                        ("cylinder", (0.007, 0.014))):
        a = S.HelmholtzResonator(position=(0.03, 0.02, 0.04), cavity_shape=shape,
                                 cavity_size=size, neck_length=0.007, neck_radius=0.003,
                                 neck_direction=(0, 1, 0))
        b = O.HelmholtzResonator(position=(0.03, 0.02, 0.04), cavity_shape=shape,
                                 cavity_size=size, neck_length=0.007, neck_radius=0.003,
                                 neck_direction=(0, 1, 0))
        na, nb = a._combined.children[1], b._combined.children[1]
        assert np.array_equal(na.p1, nb.p1) and np.array_equal(na.p2, nb.p2)
        assert na.length == nb.length


def test_nonuniform_grid_host_values(manifest):
    """NonuniformGrid coordinates, spacings and float32 stencil arrays, the
    base coefficients and the physical-distance PML profile, against the
    oracle's restatement (which the nonuniform goldens pin to the reference)."""
    from oracle import oracle as O

    specs = [("stretch", ((30, 26, 34), 1e-3, 1.04, 1.0, 1.06), dict(center_fine=True)),
             ("stretch", ((24, 28, 20), 1e-3, 1.0, 1.05, 1.03), dict(center_fine=False)),
             ("regions", ([(0.0, 0.01, 1e-3), (0.01, 0.03, 5e-4), (0.03, 0.04, 1e-3)],
                          [(0.0, 0.024, 1e-3)], [(0.0, 0.012, 1.5e-3), (0.012, 0.03, 7.5e-4)]),
              {})]
    for kind, args, kw in specs:
        mk = "from_stretch" if kind == "stretch" else "from_regions"
        g = getattr(S.NonuniformGrid, mk)(*args, **kw)
        o = getattr(O.NonuniformGrid, mk)(*args, **kw)
        for a in ("x_coords", "y_coords", "z_coords", "dx", "dy", "dz"):
            np.testing.assert_array_equal(getattr(g, a), getattr(o, a))
        assert g.min_spacing == o.min_spacing and g.shape == o.shape
        ga, oa = g.get_spacing_arrays_for_stencil(), o.get_spacing_arrays_for_stencil()
        for k in ga:
            assert ga[k].dtype == np.float32
            np.testing.assert_array_equal(ga[k], oa[k])
        pml, opml = S.PML(depth=4), O.PML(depth=4)
        pml._max_sigma = opml._max_sigma = 1234.5
        pml.order = opml.order = 3
        for c, sp in ((g.x_coords, g.dx), (g.z_coords, g.dz)):
            np.testing.assert_array_equal(pml._create_profile_nonuniform(c, sp),
                                          opml._profile_nu(c, sp, np.float32))
    g = S.NonuniformGrid.from_stretch((30, 26, 34), 1e-3, 1.04, 1.0, 1.06)
    dt, cvb, cpb = step_coefficients(g, 343.0, 1.204, 0.5)
    info = manifest["plain_nu_stretch_blocks"]
    assert (dt, cvb, cpb) == (info["dt"], info["coeff_v"], info["coeff_p"])
    assert info["uniform"] is False


def test_membrane_weights_match_oracle():
    """Mode-shape weights of the membrane sources (Bessel discs, sine
    rectangles, every normal axis, a nonuniform grid), product vs oracle
    restatement (the membrane golden pins the oracle to the reference)."""
    from oracle import oracle as O

    grids = [(S.UniformGrid((36, 32, 40), 1e-3), O.UniformGrid((36, 32, 40), 1e-3)),
             (S.NonuniformGrid.from_stretch((30, 26, 34), 1e-3, 1.04, 1.0, 1.06),
              O.NonuniformGrid.from_stretch((30, 26, 34), 1e-3, 1.04, 1.0, 1.06))]
    wf = S.GaussianPulse(position=(0, 0, 0), frequency=1000.0)
    for g, og in grids:
        for ax in "xyz":
            for mode in ((0, 1), (1, 1), (2, 2), (3, 1)):
                a = S.CircularMembraneSource(center=(0.015, 0.013, 0.017), normal_axis=ax,
                                             radius=0.0065, mode=mode, waveform=wf)
                b = O.CircularMembraneSource((0.015, 0.013, 0.017), ax, wf, 0.0065, mode=mode)
                np.testing.assert_array_equal(a.get_injection_weights(g), b.weights(og))
            for mode in ((1, 1), (1, 2), (3, 2)):
                a = S.RectangularMembraneSource(center=(0.014, 0.012, 0.016), normal_axis=ax,
                                                size=(0.01, 0.007), mode=mode, waveform=wf)
                b = O.RectangularMembraneSource((0.014, 0.012, 0.016), ax, wf, (0.01, 0.007),
                                                mode=mode)
                np.testing.assert_array_equal(a.get_injection_weights(g), b.weights(og))


def waveform_table_matches_per_step_calls(n=4000):
    """The source table evaluates a GaussianPulse over all times of a call in
    one NumPy call; every value must equal the one-element call the
    reference makes per step (elementwise ufuncs give the same bits)."""
    rng = np.random.default_rng(5)
    for f, bw, amp in ((1000.0, None, 1.0), (2500.0, 800.0, 0.7), (20000.0, 15000.0, 1.3),
                       (31000.0, None, -0.4)):
        g = S.GaussianPulse(position=(0, 0, 0), frequency=f, bandwidth=bw, amplitude=amp)
        dt = float(rng.uniform(1e-7, 2e-6))
        t, ts = float(rng.uniform(0.0, 5e-4)), []
        for _ in range(n):
            ts.append(t)
            t += dt
        ts = np.array(ts)
        per = np.array([g.waveform(np.array([x]), dt)[0] for x in ts])
        np.testing.assert_array_equal(g.waveform(ts, dt).view(np.int64), per.view(np.int64))


def test_waveform_table_matches_per_step_calls():
    waveform_table_matches_per_step_calls()


def test_differentiable_source_table_matches_per_step_calls():
    """DifferentiableSolver builds its source table in one NumPy call over the
    FP64-accumulated times t += dt; every value must equal a one-element call
    per step (checked on the CPU through a stand-in object: no device)."""
    import types

    torch = pytest.importorskip("torch")
    from strata_fdtd_gb300.adjoint import DifferentiableSolver

    for f in (1500.0, 20000.0):
        stub = types.SimpleNamespace(pulse=S.GaussianPulse(position=(0, 0, 0), frequency=f),
                                     dt=1e-3 / (343.0 * np.sqrt(3)) * 0.5, torch=torch,
                                     ext_dtype=torch.float64, dev="cpu")
        got = DifferentiableSolver.source_values(stub, 2000).numpy()
        t, per = 0.0, []
        for _ in range(2000):
            per.append(stub.pulse.waveform(np.array([t]), stub.dt)[0])
            t += stub.dt
        np.testing.assert_array_equal(got.view(np.int64), np.array(per).view(np.int64))


def test_curved_shape_constants_match_oracle_construction():
    """The host-side constants the voxeliser receives for the curved shapes
    (horn flare constants, sampled spiral and helix vertices and their radii)
    are the oracle's, computed with the same NumPy calls."""
    from oracle import oracle as O

    for prof in ("conical", "exponential", "hyperbolic", "tractrix"):
        a = S.Horn((0.0, 0.0, 0.04), (0.0, 0.0, 0.0), 0.004, 0.012, prof)
        b = O.Horn((0.0, 0.0, 0.04), (0.0, 0.0, 0.0), 0.004, 0.012, prof)
        assert a._flare() == b.k
        assert a.cutoff_frequency > 0
        np.testing.assert_allclose(a.radius_at_position([0.0, 1.0]), [0.004, 0.012], rtol=1e-12)
    for spiral in ("logarithmic", "archimedean"):
        for prof in ("exponential", "linear", "hyperbolic"):
            a = S.SpiralHorn((0.03, 0.03), 0.003, 0.006, 0.008, 0.022, 2.3, 0.02, prof, spiral)
            b = O.SpiralHorn((0.03, 0.03), 0.003, 0.006, 0.008, 0.022, 2.3, 0.02, prof, spiral)
            np.testing.assert_array_equal(a.path_2d, b.path)
            np.testing.assert_array_equal(a.radii, b.radii)
            assert len(a.path_2d) == max(200, int(100 * 2.3))  # 229: int() truncates
            assert a.program()[1] == 1 + len(a.path_2d)
    a = S.HelicalTube((0.025, 0.025, 0.004), 0.013, 0.003, 0.005, 0.012, 2.0)
    b = O.HelicalTube((0.025, 0.025, 0.004), 0.013, 0.003, 0.005, 0.012, 2.0)
    np.testing.assert_array_equal(a.path_3d, b.path)
    np.testing.assert_array_equal(a.tube_radii, b.radii)
    assert a.helix.total_height == pytest.approx(0.024)
    pts = np.random.default_rng(1).uniform(0, 0.05, (200, 3))
    np.testing.assert_array_equal(S.distance_to_polyline(pts, a.path_3d),
                                  O._polyline_distance(pts, b.path))
    for bad in (dict(r1=0.0, r2=0.0), dict(r1=-1.0, r2=0.1)):
        with pytest.raises(ValueError):
            S.Cone((0, 0, 0), (0, 0, 1), **bad)
    with pytest.raises(ValueError):
        S.Horn((0, 0, 0), (0, 0, 1), 0.1, 0.2, "parabolic")
    with pytest.raises(ValueError):
        S.SmoothUnion(S.Sphere((0, 0, 0), 1.0), S.Sphere((1, 0, 0), 1.0), 0.0)


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every ctypes mirror of a struct in include/sf_gb300.h has the C
    compiler's size and field offsets (a program built from the header by
    the host compiler prints them)."""
    import shutil
    import subprocess

    from strata_fdtd_gb300 import adjoint as A

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    mirrors = {"sf_grid_desc": _native.SfGridDesc, "sf_source": _native.SfSource,
               "sf_pole": _native.SfPole, "sf_plane_bc": _native.SfPlaneBC,
               "sf_sdf_node": _native.SfSdfNode, "sf_device_info_t": _native.SfDeviceInfo,
               "sf_diff_desc": A._Desc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sf_gb300.h"',
             'int main(void) {']
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in
               subprocess.run([str(exe)], check=True, capture_output=True,
                              text=True).stdout.splitlines())
    for cname, cls in mirrors.items():
        assert int(got[f"{cname} size"]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname} {fname}"]) == getattr(cls, fname).offset, (cname, fname)


def test_unit_decay_ranges():
    """The differentiable solve's unit-decay ranges: the longest run of
    indices whose decay and both neighbours' are exactly 1 (past either end
    counts as 1)."""
    from strata_fdtd_gb300.adjoint import _unit_range

    assert _unit_range(np.array([0.5, 0.9, 1, 1, 1, 1, 0.9, 0.5])) == (3, 5)
    assert _unit_range(np.ones(5)) == (0, 5)
    assert _unit_range(np.array([0.5, 1.0, 0.5])) == (0, 0)
    assert _unit_range(np.array([1, 1, 0.5, 1, 1, 1, 1])) == (4, 7)
    assert _unit_range(np.array([1, 1, 1, 0.5, 1, 1])) == (0, 2)
