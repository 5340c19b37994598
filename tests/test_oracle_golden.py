"""Pin the CPU oracle against the reference's own outputs (tests/golden/).

The oracle (oracle/sf_oracle.c + oracle/oracle.py) is the parity checker for
every GPU test, so it is checked first: bit-exact final fields and probe
traces for the plain native path, the ADE order, SDF voxelisation, the
rigid-face lists and the host-side values (waveform, pole coefficients, PML
profiles and decays).  CPU only.
"""
import numpy as np
import pytest

import cases as C
from conftest import golden, sha256
from oracle import oracle as O

API = O.make_api()
SMALL_PLAIN = [k for k, v in C.PLAIN_CASES.items() if not v.get("big")]


def _run(case, step_by_step):
    s = C.build_case(API, case)
    if step_by_step:
        for _ in range(case["steps"]):
            s.step()
    else:
        s.run_steps(case["steps"])
    return s


def _check(s, key, manifest):
    info = manifest[key]
    g = golden(key)
    for f in ("p", "vx", "vy", "vz"):
        arr = getattr(s, f)
        if f"field__{f}" in g.files:
            np.testing.assert_array_equal(arr, g[f"field__{f}"], err_msg=f"{key} {f}")
        assert sha256(arr) == info[f"sha_{f}"], f"{key}: {f} differs from the reference"
    for name in g["probe_names"]:
        np.testing.assert_array_equal(s.get_probe_data()[str(name)], g[f"trace__{name}"])


@pytest.mark.parametrize("name", SMALL_PLAIN)
def test_plain_fused_loop_matches_reference(name, manifest):
    _check(_run(C.PLAIN_CASES[name], step_by_step=False), "plain_" + name, manifest)


@pytest.mark.parametrize("name", ["mics_geom", "mics_directional"])
def test_microphones_match_reference(name, manifest):
    """Omni microphones through the native batch kernel's float32 weights;
    with directional ones present, every microphone through the reference's
    Python path (FP64 weights, staggered clamped velocity interpolation,
    pattern combination, a custom gain)."""
    case = C.PLAIN_CASES[name]
    s = _run(case, step_by_step=True)
    _check(s, "plain_" + name, manifest)
    g = golden("plain_" + name)
    mics = s.get_mic_data()
    assert len(mics) == len(case["mics"])
    for mic, tr in mics.items():
        np.testing.assert_array_equal(tr, g[f"mic__{mic}"])


@pytest.mark.parametrize("name", ["c1_tiny", "blocks_odd", "plane_yz_geom"])
def test_plain_kernel_by_kernel_matches_reference(name, manifest):
    _check(_run(C.PLAIN_CASES[name], step_by_step=True), "plain_" + name, manifest)


@pytest.mark.parametrize("name", list(C.ADE_CASES))
def test_ade_matches_reference_kernels(name, manifest):
    s = _run(C.ADE_CASES[name], step_by_step=True)
    _check(s, "ade_" + name, manifest)
    g = golden("ade_" + name)
    jd = [e["J"] for e in s._ade["debye"]]
    if jd:
        np.testing.assert_array_equal(np.concatenate(jd), g["ade_ade_J_debye"])
    jl = [e["J"] for e in s._ade["lorentz"]]
    if jl:
        np.testing.assert_array_equal(np.concatenate(jl), g["ade_ade_J_lorentz"])


def test_materialized_geometry_ids_match_reference():
    """MaterializedGeometry (geometry/material_assignment.py:133-171) through
    the oracle's set_geometry: mask and material ids equal the reference's."""
    case = C.ADE_CASES["materialized_sdf"]
    s = C.build_case(API, case)
    g = golden("ade_materialized_sdf")
    geom = np.unpackbits(g["geometry"])[: s.geometry.size].reshape(s.geometry.shape)
    np.testing.assert_array_equal(s.geometry, geom.astype(bool))
    np.testing.assert_array_equal(s._material_id, g["material_id"])
    assert sorted(s._materials) == [1, 2, 3]


def test_fp64_run_is_close_to_fp32():
    case = C.PLAIN_CASES["blocks_odd"]
    a = _run(case, False)
    kw = dict(grid=O.UniformGrid(case["shape"], case["res"]), c=343.0, rho=1.204,
              courant=case["courant"], precision="f64")
    b = O.FDTDSolver(**kw)
    b.add_boundary(O.PML(**case["pml"]))
    b.set_geometry(C._mask_blocks(case["shape"], case["geometry"]["seed"]))
    for kind, pos, f, amp in case["sources"]:
        b.add_source(O.GaussianPulse(position=pos, frequency=f, amplitude=amp))
    b.run_steps(case["steps"])
    rel = np.linalg.norm(a.p.astype(np.float64) - b.p) / np.linalg.norm(b.p)
    assert 0 < rel < 1e-4


@pytest.mark.parametrize("name", list(C.VOXEL_CASES))
def test_voxelize_matches_reference(name):
    shape, res, which = C.VOXEL_CASES[name]
    if which in ("bookshelf", "cabinet"):
        pytest.skip("the oracle restates shapes, not the loudspeaker builder")
    mask = C.sdf_tree(API, which).voxelize(O.UniformGrid(shape, res))
    ref = np.unpackbits(golden("voxel")["mask__" + name])[: mask.size].reshape(shape)
    np.testing.assert_array_equal(mask, ref.astype(bool))


@pytest.mark.parametrize("name", ["blocks_odd", "plane_yz_geom", "sdf_geometry"])
def test_boundary_face_lists_match_reference(name):
    g = golden("plain_" + name)
    shape = C.PLAIN_CASES[name]["shape"]
    geom = np.unpackbits(g["geometry"])[: int(np.prod(shape))].reshape(shape).astype(bool)
    for axis, key in enumerate(("bc_vx", "bc_vy", "bc_vz")):
        np.testing.assert_array_equal(O.boundary_faces(geom, axis), g[key])


def test_host_values_match_reference():
    h = golden("host_values")
    for f in (1000, 2000, 20000):
        g = O.GaussianPulse(position=(0, 0, 0), frequency=float(f),
                            bandwidth=15000.0 if f == 20000 else None, amplitude=1.3)
        dt = 0.5 * (1e-3 / (343.0 * np.sqrt(3)))
        vals = [g.waveform(np.array([t]), dt)[0] for t in h[f"wave_t__{f}"]]
        np.testing.assert_array_equal(np.array(vals), h[f"wave__{f}"])
    for row in h["pole_rows"]:
        dt, kind = row[0], int(row[1])
        if kind == 0:
            p = O.Pole(O.PoleType.DEBYE, delta_chi=row[3], target="density", tau=row[2])
            assert p.fdtd_coefficients(dt) == tuple(row[4:6])
        else:
            p = O.Pole(O.PoleType.LORENTZ, delta_chi=0.2, target="modulus", omega_0=row[2],
                       gamma=row[3])
            assert p.fdtd_coefficients(dt) == tuple(row[4:7])
    for n in (100, 37, 400):
        sig = h[f"sigma__{n}"]
        out = np.zeros(n, dtype=np.float32)
        O.lib().orc_pml_decay_f32(sig.ctypes.data, n, float(np.float32(h[f"dt__{n}"][0])),
                                 out.ctypes.data)
        np.testing.assert_array_equal(out, h[f"decay__{n}"])
