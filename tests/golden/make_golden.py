#!/usr/bin/env python3
"""Generate the golden vectors under tests/golden/ by running the reference.

Runs only where the reference tree exists (REF_ROOT, default
/root/reference) and after ``make -C oracle ref`` has compiled the
reference's own pybind11 module from its sources into oracle/_ref/.  The GPU
box never runs this file; it only reads the .npz fixtures it writes.

How the reference is imported: its package imports the native module under
three names (core/solver.py:82-92, boundaries/_boundaries.py:62-69) while the
build installs one, so the module is loaded once and aliased under all three;
``h5py`` (needed only by its io/ package at import time) is stubbed.

What is stored:
  plain_<case>.npz  reference FDTDSolver(backend="native"), step for step:
                    probe traces, final p/vx/vy/vz (full arrays for small
                    cases, sha256 for all), coefficients, PML decays, the
                    geometry mask and the BoundaryCells index lists.
  ade_<case>.npz    reference ADE kernels in _step_python_uniform's order
                    (core/solver.py:2135-2193) -- its native step drops ADE.
  voxel.npz         SDFPrimitive.voxelize masks, bit-packed.
  host_values.npz   GaussianPulse.waveform samples, Pole.fdtd_coefficients,
                    PML sigma profiles and decays.
"""
from __future__ import annotations

import glob
import hashlib
import importlib.util
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")
sys.path.insert(0, HERE)
import cases as C  # noqa: E402


def load_reference():
    sys.path.insert(0, os.path.join(REF_ROOT, "src"))
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    so = glob.glob(os.path.join(REPO, "oracle", "_ref", "_kernels*.so"))
    if not so:
        raise SystemExit("build the reference module first: make -C oracle ref")
    spec = importlib.util.spec_from_file_location("_kernels", so[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    for name in ("strata_fdtd._kernels", "strata_fdtd.core._kernels",
                 "strata_fdtd.boundaries._kernels"):
        sys.modules[name] = mod
    import strata_fdtd as sf
    from strata_fdtd.geometry import material_assignment, resonator, sdf
    from strata_fdtd.materials import base
    api = types.SimpleNamespace(
        FDTDSolver=sf.FDTDSolver, UniformGrid=sf.UniformGrid, PML=sf.PML,
        NonuniformGrid=sys.modules["strata_fdtd.core.grid"].NonuniformGrid,
        ABCFirstOrder=sys.modules["strata_fdtd.boundaries"].ABCFirstOrder,
        RadiationImpedance=sf.RadiationImpedance,
        CircularMembraneSource=sys.modules["strata_fdtd.core.solver"].CircularMembraneSource,
        RectangularMembraneSource=sys.modules["strata_fdtd.core.solver"].RectangularMembraneSource,
        GaussianPulse=sf.GaussianPulse, Box=sdf.Box, Sphere=sdf.Sphere,
        Cylinder=sdf.Cylinder, Union=sdf.Union, Intersection=sdf.Intersection,
        Difference=sdf.Difference, HelmholtzResonator=resonator.HelmholtzResonator,
        Cone=sdf.Cone, Horn=sdf.Horn, SpiralHorn=sdf.SpiralHorn, HelicalTube=sdf.HelicalTube,
        SmoothUnion=sdf.SmoothUnion, SmoothIntersection=sdf.SmoothIntersection,
        SmoothDifference=sdf.SmoothDifference,
        LoudspeakerEnclosure=sys.modules["strata_fdtd.geometry.loudspeaker"].LoudspeakerEnclosure,
        bookshelf_speaker=sys.modules["strata_fdtd.geometry.loudspeaker"].bookshelf_speaker,
        tower_speaker=sys.modules["strata_fdtd.geometry.loudspeaker"].tower_speaker,
        Pole=base.Pole, PoleType=base.PoleType, SimpleMaterial=base.SimpleMaterial,
        MaterializedGeometry=material_assignment.MaterializedGeometry,
        kernels=mod, solver_module=sys.modules["strata_fdtd.core.solver"])
    assert api.solver_module.has_native_kernels()
    return api


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ade_step_native(self):
    """Reference ADE kernels in _step_python_uniform's order
    (core/solver.py:2135-2193), each through the reference's own helper; on a
    nonuniform grid _step_python_nonuniform's order (2195-2283) with the
    native nonuniform velocity and pressure updates of _step_native_nonuniform
    (2104-2126).  The ADE helpers pick their own native calls (uniform-dx
    corrections, compute_divergence_nonuniform on a nonuniform grid)."""
    K = sys.modules["strata_fdtd.core._kernels"]
    uniform = self._grid.is_uniform
    self._update_ade_density_poles()
    if uniform:
        K.update_velocity(self.p, self.vx, self.vy, self.vz, self._coeff_v)
    else:
        K.update_velocity_nonuniform(self.p, self.vx, self.vy, self.vz, self._native_grid_data,
                                     self._coeff_v_base)
    self._apply_ade_velocity_correction()
    if self._boundary_cells is not None:
        K.apply_rigid_boundaries(self.vx, self.vy, self.vz, self._boundary_cells)
    self._update_ade_modulus_poles()
    if uniform:
        K.update_pressure(self.p, self.vx, self.vy, self.vz, self.geometry, self._coeff_p)
    else:
        K.update_pressure_nonuniform(self.p, self.vx, self.vy, self.vz, self.geometry,
                                     self._native_grid_data, self._coeff_p_base)
    self._apply_ade_pressure_correction()
    self.p[~self.geometry] = 0.0


def fill_ade_native(self, K):
    """Rebuild _ade_native_data as _initialize_ade_native (core/solver.py:
    2996-3083) intends.  The reference fills it through element writes and
    .append() on pybind11 def_readwrite std::vector members, which act on
    temporary Python copies, so its native ADE tables stay empty
    (debye_poles == [], rho_inf == [0.0, ...]).  Whole-list assignment is
    used here instead; the values and the field numbering are the same."""
    data = K.ADEMaterialData()
    top = max(self._materials)
    rho = [0.0] * (top + 1)
    kin = [0.0] * (top + 1)
    debye, lorentz = [], []
    for mid, mat in self._materials.items():
        rho[mid], kin[mid] = float(mat.rho_inf), float(mat.K_inf)
        for pole in mat.poles:
            if pole.is_debye:
                e = K.ADEDebyePole()
                co = K.DebyePoleCoeffs()
                co.alpha, co.beta = (float(v) for v in pole.fdtd_coefficients(self.dt))
                e.field_index = len(debye)
                debye.append(e)
            else:
                e = K.ADELorentzPole()
                co = K.LorentzPoleCoeffs()
                co.a, co.b, co.d = (float(v) for v in pole.fdtd_coefficients(self.dt))
                e.field_index = len(lorentz)
                lorentz.append(e)
            e.material_id = mid
            e.target = 0 if pole.target == "density" else 1
            e.coeffs = co
    data.rho_inf, data.K_inf = rho, kin
    data.debye_poles, data.lorentz_poles = debye, lorentz
    data.n_debye_fields, data.n_lorentz_fields = len(debye), len(lorentz)
    assert len(data.debye_poles) == len(debye) and data.rho_inf == [float(np.float32(r)) for r in rho]
    self._ade_native_data = data


def run_case(api, name, case, ade, manifest):
    t0 = time.time()
    solver = C.build_case(api, case)
    if ade:
        solver._initialize_ade_fields()
        fill_ade_native(solver, api.kernels)
        solver._step_native = types.MethodType(ade_step_native, solver)
        solver._step_native_nonuniform = types.MethodType(ade_step_native, solver)
    for _ in range(case["steps"]):
        solver.step()
    out = {}
    traces = solver.get_probe_data()
    out["probe_names"] = np.array(list(traces.keys()))
    for pname, tr in traces.items():
        out[f"trace__{pname}"] = tr
    for mic_name, mic in getattr(solver, "_microphones", {}).items():
        out[f"mic__{mic_name}"] = mic.get_waveform()
    uniform = solver.grid.is_uniform
    info = dict(steps=case["steps"], dt=float(solver.dt),
                coeff_v=float(solver._coeff_v if uniform else solver._coeff_v_base),
                coeff_p=float(solver._coeff_p if uniform else solver._coeff_p_base),
                time=float(solver._time), uniform=bool(uniform))
    for f in ("p", "vx", "vy", "vz"):
        arr = getattr(solver, f)
        info[f"sha_{f}"] = sha(arr)
        info[f"l2_{f}"] = float(np.sqrt(np.sum(arr.astype(np.float64) ** 2)))
        if case.get("store_fields"):
            out[f"field__{f}"] = arr
    info["sha_geometry"] = sha(solver.geometry)
    if not case.get("big"):
        out["geometry"] = np.packbits(solver.geometry.ravel())
    if solver._boundary_cells is not None and not case.get("big"):
        out["bc_vx"] = np.asarray(solver._boundary_cells.vx_indices, dtype=np.int32)
        out["bc_vy"] = np.asarray(solver._boundary_cells.vy_indices, dtype=np.int32)
        out["bc_vz"] = np.asarray(solver._boundary_cells.vz_indices, dtype=np.int32)
    if ade:
        for key in ("_ade_J_debye", "_ade_J_lorentz", "_ade_J_lorentz_prev"):
            arr = getattr(solver, key)
            info[f"sha{key}"] = sha(arr)
            out[f"ade{key}"] = arr
        out["material_id"] = solver._material_id
    if case.get("probes") == "c2":
        info["probes"] = [(p.name, list(p.position)) for p in solver._probes.values()]
    info["seconds"] = round(time.time() - t0, 2)
    manifest[("ade_" if ade else "plain_") + name] = info
    np.savez_compressed(os.path.join(HERE, ("ade_" if ade else "plain_") + name + ".npz"), **out)
    print(f"{name}: {info['seconds']} s", flush=True)


def python_backend_run(api, name, case, manifest):
    """The same ADE case on backend="python" (FP64-coefficient NumPy
    arithmetic), kept only to report how far the FP32 native order lies from
    the reference's python path."""
    c = dict(case)
    solver = C.build_case(api, c)
    solver._use_native = False
    solver._initialize_ade_fields()
    for _ in range(case["steps"]):
        solver._step_python()
        for b in solver._boundaries:
            b.apply_velocity(solver)
        for b in solver._boundaries:
            b.apply_pressure(solver)
        solver._inject_sources()
        solver._record_probes()
        solver._time += solver.dt
    out = {f"trace__{k}": v for k, v in solver.get_probe_data().items()}
    if case.get("store_fields"):
        out["field__p"] = solver.p
    np.savez_compressed(os.path.join(HERE, f"pyade_{name}.npz"), **out)


def voxel_cases(api, manifest):
    out = {}
    for name, (shape, res, which) in C.VOXEL_CASES.items():
        grid = api.UniformGrid(shape=shape, resolution=res)
        mask = C.sdf_tree(api, which).voxelize(grid)
        out[f"mask__{name}"] = np.packbits(mask.ravel())
        manifest[f"voxel_{name}"] = dict(shape=list(shape), res=res, inside=int(mask.sum()),
                                         sha=sha(mask))
    np.savez_compressed(os.path.join(HERE, "voxel.npz"), **out)


def host_values(api, manifest):
    out = {}
    K = api.kernels
    # GaussianPulse.waveform at the solver's accumulated times (FP64 _time += dt)
    for f, bw in ((1000.0, None), (2000.0, None), (20000.0, 15000.0)):
        g = api.GaussianPulse(position=(0, 0, 0), frequency=f, bandwidth=bw, amplitude=1.3)
        dt = 0.5 * (1e-3 / (343.0 * np.sqrt(3)))
        t, vals, times = 0.0, [], []
        for _ in range(600):
            vals.append(g.waveform(np.array([t]), dt)[0])
            times.append(t)
            t += dt
        out[f"wave__{int(f)}"] = np.array(vals)
        out[f"wave_t__{int(f)}"] = np.array(times)
    # Pole.fdtd_coefficients (materials/base.py:157-188)
    rows = []
    for dt in (8.416184682064516e-07, 1.5e-6):
        for tau in (1e-5, 1e-4, 1e-3):
            p = api.Pole(pole_type=api.PoleType.DEBYE, delta_chi=0.37, target="density", tau=tau)
            rows.append([dt, 0, tau, 0.37, *p.fdtd_coefficients(dt), 0.0])
        for w0, gam in ((2 * np.pi * 500.0, 10.0), (2 * np.pi * 9000.0, 4000.0)):
            p = api.Pole(pole_type=api.PoleType.LORENTZ, delta_chi=0.2, target="modulus",
                         omega_0=w0, gamma=gam)
            rows.append([dt, 1, w0, gam, *p.fdtd_coefficients(dt)])
    out["pole_rows"] = np.array(rows)
    # PML sigma profiles and decays (boundaries/_boundaries.py:166-255, pml.cpp:13-45)
    for n, depth, res, courant in ((100, 10, 1e-3, 0.5), (37, 6, 2e-3, 0.9), (400, 16, 1e-3, 0.5)):
        s = api.FDTDSolver(shape=(n, 4, 4), resolution=res, c=343.0, rho=1.204,
                           courant=courant, backend="native")
        pml = api.PML(depth=depth, axis="x")
        s.add_boundary(pml)
        out[f"sigma__{n}"] = pml._sigma_x
        out[f"dt__{n}"] = np.array([s.dt])
        lib = np.ctypeslib.load_library("libref_kernels", os.path.join(REPO, "oracle", "_ref"))
        import ctypes
        lib.ref_pml_create.restype = ctypes.c_void_p
        lib.ref_pml_create.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3 + [ctypes.c_float]
        h = lib.ref_pml_create(pml._sigma_x.ctypes.data, None, None, n, 4, 4, float(s.dt))
        dec = np.zeros(n, dtype=np.float32)
        lib.ref_pml_decay.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.ref_pml_decay(ctypes.c_void_p(h), 0, dec.ctypes.data)
        lib.ref_pml_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_pml_destroy(ctypes.c_void_p(h))
        out[f"decay__{n}"] = dec
    np.savez_compressed(os.path.join(HERE, "host_values.npz"), **out)


def analysis_values(api, manifest):
    """Host-side quantities around the solve, from the reference's own code:
    A/C weighting filters and sound levels (analysis/weighting.py), the
    frequency-domain material properties (materials/base.py:215-507) and the
    horn flare functions (geometry/sdf.py:1039-1083)."""
    import strata_fdtd.analysis.weighting as W

    out = {}
    dt = 0.5 * (1e-3 / (343.0 * np.sqrt(3)))
    for fs in (48000.0, 1.0 / dt):
        for w in ("A", "C"):
            out[f"sos_{w}__{int(fs)}"] = W.get_weighting_sos(w, fs)
    rng = np.random.default_rng(5)
    fs = 48000.0
    tt = np.arange(4800) / fs
    wave = (0.3 * np.sin(2 * np.pi * 90 * tt) + 0.2 * np.sin(2 * np.pi * 1000 * tt)
            + 0.05 * np.sin(2 * np.pi * 9000 * tt) + 0.01 * rng.standard_normal(tt.size))
    wave = wave.astype(np.float32)
    out["level_wave"] = wave
    for w in ("A", "C", None):
        key = w or "Z"
        weighted = W.apply_weighting(wave, fs, w)
        out[f"weighted__{key}"] = weighted[::8]  # every 8th sample kept
        out[f"spl__{key}"] = np.array([W.calculate_spl(weighted)])
        out[f"leq_005__{key}"] = np.array([W.calculate_leq(weighted, fs, 0.05)])
        for tc in ("fast", "slow", "impulse"):
            out[f"twl_{tc}__{key}"] = W.calculate_time_weighted_level(weighted, fs, tc)[::16]
    mat = api.SimpleMaterial(name="m", _rho=1.3, _c=330.0, _poles=[
        api.Pole(pole_type=api.PoleType.DEBYE, delta_chi=0.4, target="density", tau=2e-4),
        api.Pole(pole_type=api.PoleType.LORENTZ, delta_chi=0.25, target="modulus",
                 omega_0=2 * np.pi * 2000.0, gamma=900.0)])
    om = 2 * np.pi * np.array([50.0, 300.0, 1000.0, 2000.0, 4500.0, 12000.0])
    out["mat_omega"] = om
    for name in ("effective_density", "effective_modulus", "wavenumber", "phase_velocity",
                 "group_velocity", "impedance", "attenuation", "attenuation_db_per_meter"):
        out[f"mat_{name}"] = np.asarray(getattr(mat, name)(om))
    out["mat_reflection"] = mat.reflection_coefficient(om, 415.0)
    out["mat_absorption"] = mat.absorption_coefficient(om, 415.0)
    out["mat_scalars"] = np.array([mat.c_inf, mat.Z_inf,
                                   api.SimpleMaterial.from_impedance("w", 998.0, 1.48e6).c_inf])
    ts = np.linspace(0, 1, 11)
    for prof in ("conical", "exponential", "hyperbolic", "tractrix"):
        h = api.Horn((0.0, 0.0, 0.05), (0.0, 0.0, 0.0), 0.006, 0.02, prof)
        out[f"horn_{prof}"] = np.concatenate([[h.cutoff_frequency], h.radius_at_position(ts)])
    # the material library's poles and the models' analytic responses
    # (materials/library.py, porous.py, solids.py, resonators.py)
    import strata_fdtd.materials as MM

    def pole_rows(mat):
        return np.array([[0 if p.is_debye else 1, p.delta_chi, p.tau or 0.0, p.omega_0 or 0.0,
                          p.gamma or 0.0, 0 if p.target == "density" else 1]
                         for p in mat.poles]).reshape(-1, 6)

    for name in MM.list_materials():
        out[f"lib__{name}"] = pole_rows(MM.get_material(name))
    extra = {
        "helmholtz": MM.HelmholtzResonator(name="h", neck_radius=0.02, neck_length=0.04,
                                           cavity_volume=0.015, loss_factor=0.12),
        "membrane": MM.MembraneAbsorber(name="m", surface_density=4.2, cavity_depth=0.15),
        "perforated": MM.PerforatedPanel(name="p", hole_diameter=0.003, plate_thickness=0.012,
                                         perforation_ratio=0.15, cavity_depth=0.2),
        "quarter": MM.QuarterWaveResonator(name="q", length=0.858, diameter=0.1,
                                           loss_factor=0.08, n_modes=4),
        "porous_thick": MM.PorousMaterial(name="pt", flow_resistivity=18000, porosity=0.97,
                                          tortuosity=1.05, viscous_length=90e-6,
                                          thermal_length=180e-6, thickness=0.05, num_poles=8),
    }
    for key, mat in extra.items():
        out[f"model__{key}"] = pole_rows(mat)
    om = 2 * np.pi * np.array([63.0, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0])
    pt = extra["porous_thick"]
    tube = MM.ImpedanceTube(length=0.5, diameter=0.1, mic_spacing=0.05, sample_distance=0.1)
    out["model_resp"] = np.concatenate([
        pt.jca_impedance(om), pt.surface_impedance(om), pt.surface_impedance(om, backing=900.0),
        pt.absorption_coefficient_layer(om), tube.absorption_coefficient(pt, om),
        tube.absorption_coefficient(MM.MDF_MEDIUM, om), MM.MDF_MEDIUM.loss_factor_spectrum(om),
        MM.SORBOTHANE.quality_factor(om), extra["helmholtz"].absorption_analytical(om),
        extra["perforated"].impedance_analytical(om)]).astype(complex)
    fit = pt.validate_pole_fit(om)
    out["model_scalars"] = np.array([
        extra["helmholtz"].resonance_frequency, extra["helmholtz"].quality_factor_theoretical,
        extra["membrane"].resonance_frequency, extra["perforated"].resonance_frequency,
        extra["quarter"].fundamental_frequency, MM.MDF_MEDIUM.c_longitudinal,
        tube.max_frequency, tube.min_frequency, fit["density_max_error"],
        fit["modulus_mean_error"]])
    # a cabinet's membrane sources and absorber regions (geometry/loudspeaker.py)
    enc = C.loudspeaker_cabinet(api, waveform=api.GaussianPulse(position=(0, 0, 0),
                                                               frequency=400.0))
    out["cab_sources"] = np.array([list(s.center) + [s.radius, "xyz".index(s.normal_axis),
                                                     *s.mode] for s in enc.get_membrane_sources()])
    out["cab_regions"] = np.array([list(b.center) + list(b.size) + [mid]
                                   for b, mid in enc.get_material_regions()])
    t = api.tower_speaker(0.22, 0.3, 0.9, 0.17, 0.13, 0.025)
    out["tower_inside_4mm"] = np.array([int(t.build().voxelize(
        api.UniformGrid(shape=(55, 75, 225), resolution=4e-3)).sum())])
    # source-signal processing (dsp/): filters, crossovers, delay, EQ over a
    # pulse sampled at 48 kHz
    import strata_fdtd.dsp as D

    for key, wf in C.dsp_waveforms(api, D).items():
        out[f"dsp__{key}"] = np.asarray(wf.waveform(np.arange(1500) / 48000.0, 1 / 48000.0))
    # weighting responses (analysis/weighting.py:304-333) and distances to a
    # helix (geometry/paths.py:296-344)
    for w in ("A", "C", None):
        f, mag = W.weighting_response(w, 48000.0, 512)
        out[f"wresp__{w or 'Z'}"] = np.stack([f, mag])
    from strata_fdtd.geometry.paths import distance_to_helix

    pts = np.random.default_rng(11).uniform(-0.05, 0.15, size=(64, 3))
    out["helix_dist"] = np.concatenate([
        distance_to_helix(pts, (0.05, 0.05, 0.0), 0.04, 0.03, 2.5),
        distance_to_helix(pts, (0.0, 0.02, 0.01), 0.02, 0.05, 0.7)])
    out["helix_pts"] = pts
    np.savez_compressed(os.path.join(HERE, "analysis_values.npz"), **out)
    manifest["analysis_values"] = dict(keys=sorted(out))


def legacy_io(api, manifest):
    """The reference's legacy result files (io/legacy.py, loaded from its
    file: the io package imports h5py): the array exporters on fixed
    arrays, and a small solve with pressure and velocity snapshots exported
    whole.  Stored: each call's returned metadata and every file's bytes
    (paths inside the JSON files written as <dir>)."""
    import tempfile

    spec = importlib.util.spec_from_file_location(
        "ref_legacy", os.path.join(REF_ROOT, "src", "strata_fdtd", "io", "legacy.py"))
    L = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(L)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        meta, files = C.legacy_array_exports(L, d)
    for k, v in meta.items():
        out[f"meta__arrays__{k}"] = np.array(v)
    for k, v in files.items():
        out[f"file__arrays__{k}"] = np.frombuffer(v, dtype=np.uint8)
    case = C.LEGACY_CASE
    solver = C.build_case(api, case)
    solver.enable_snapshots(case["snapshot_interval"], capture_velocity=True)
    for _ in range(case["steps"]):
        solver.step()
    with tempfile.TemporaryDirectory() as d:
        meta, files = C.legacy_solve_exports(L, solver, d)
    for k, v in meta.items():
        out[f"meta__solve__{k}"] = np.array(v)
    for k, v in files.items():
        out[f"file__solve__{k}"] = np.frombuffer(v, dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "legacy_io.npz"), **out)
    manifest["legacy_io"] = dict(keys=sorted(out))


def main():
    only = set(sys.argv[1:])
    api = load_reference()
    mpath = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(mpath)) if os.path.exists(mpath) else {}
    manifest["_generator"] = dict(numpy=np.__version__, python=sys.version.split()[0],
                                  reference="rjwalters/strata-fdtd (native _kernels 0.1.0)")
    for name, case in C.PLAIN_CASES.items():
        if not only or name in only:
            run_case(api, name, case, False, manifest)
    for name, case in C.ADE_CASES.items():
        if not only or name in only:
            run_case(api, name, case, True, manifest)
            python_backend_run(api, name, case, manifest)
    if not only or "voxel" in only:
        voxel_cases(api, manifest)
    if not only or "host" in only:
        host_values(api, manifest)
    if not only or "analysis" in only:
        analysis_values(api, manifest)
    if not only or "legacy" in only:
        legacy_io(api, manifest)
    with open(mpath, "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
