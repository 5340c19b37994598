"""Host-side quantities around the solve against values the reference's own
code produced (tests/golden/analysis_values.npz, tests/golden/make_golden.py
``analysis``): A/C frequency weighting and sound levels (analysis/
weighting.py), the frequency-domain material properties (materials/
base.py:215-507), the horn flare functions (geometry/sdf.py:1039-1083), and
the microphone's level, WAV and host-record methods on a recorded waveform.
Tolerance: rel 1e-12 (the same SciPy and NumPy calls; only the filter gain
is formed in a different expression)."""
import wave

import numpy as np
import pytest

import strata_fdtd_gb300 as S
from conftest import golden
from strata_fdtd_gb300 import weighting as W

pytest.importorskip("scipy")
G = golden("analysis_values")
RTOL = 1e-12


def test_weighting_filters_and_levels_match_reference():
    dt = 0.5 * (1e-3 / (343.0 * np.sqrt(3)))
    for fs in (48000.0, 1.0 / dt):
        for w in ("A", "C"):
            np.testing.assert_allclose(W.get_weighting_sos(w, fs), G[f"sos_{w}__{int(fs)}"],
                                       rtol=RTOL, atol=1e-300)
    wave_ = G["level_wave"]
    fs = 48000.0
    for w in ("A", "C", None):
        key = w or "Z"
        weighted = W.apply_weighting(wave_, fs, w)
        np.testing.assert_allclose(weighted[::8], G[f"weighted__{key}"], rtol=1e-9, atol=1e-15)
        assert W.calculate_spl(weighted) == pytest.approx(float(G[f"spl__{key}"][0]), rel=RTOL)
        assert W.calculate_leq(weighted, fs, 0.05) == pytest.approx(
            float(G[f"leq_005__{key}"][0]), rel=RTOL)
        for tc in ("fast", "slow", "impulse"):
            np.testing.assert_allclose(W.calculate_time_weighted_level(weighted, fs, tc)[::16],
                                       G[f"twl_{tc}__{key}"], rtol=1e-10)
    assert W.calculate_spl(np.zeros(8)) == -np.inf
    with pytest.raises(ValueError):
        W.get_weighting_sos("B", fs)


def test_material_properties_match_reference():
    mat = S.SimpleMaterial(name="m", _rho=1.3, _c=330.0, _poles=[
        S.Pole(S.PoleType.DEBYE, delta_chi=0.4, target="density", tau=2e-4),
        S.Pole(S.PoleType.LORENTZ, delta_chi=0.25, target="modulus", omega_0=2 * np.pi * 2000.0,
               gamma=900.0)])
    om = G["mat_omega"]
    for name in ("effective_density", "effective_modulus", "wavenumber", "phase_velocity",
                 "group_velocity", "impedance", "attenuation", "attenuation_db_per_meter"):
        np.testing.assert_allclose(getattr(mat, name)(om), G[f"mat_{name}"], rtol=1e-9,
                                   err_msg=name)
    np.testing.assert_allclose(mat.reflection_coefficient(om, 415.0), G["mat_reflection"],
                               rtol=1e-12)
    np.testing.assert_allclose(mat.absorption_coefficient(om, 415.0), G["mat_absorption"],
                               rtol=1e-12)
    want = G["mat_scalars"]
    assert mat.c_inf == want[0] and mat.Z_inf == want[1]
    assert S.SimpleMaterial.from_impedance("w", 998.0, 1.48e6).c_inf == want[2]
    assert isinstance(mat, S.AcousticMaterial)
    assert mat.n_density_poles() == 1 and mat.n_modulus_poles() == 1
    assert "Poles: 2 (1 density, 1 modulus)" in mat.summary()


def test_weighting_response_and_helix_distance_match_reference():
    from strata_fdtd_gb300.analysis import weighting_response
    from strata_fdtd_gb300.geometry import distance_to_helix

    for w in ("A", "C", None):
        f, mag = weighting_response(w, 48000.0, 512)
        np.testing.assert_allclose(f, G[f"wresp__{w or 'Z'}"][0], rtol=RTOL)
        np.testing.assert_allclose(mag, G[f"wresp__{w or 'Z'}"][1], rtol=1e-9, atol=1e-9)
    f, mag = weighting_response("A", 48000.0, 4800)
    assert f[200] == 1000.0 and abs(mag[200]) < 0.05  # 0 dB at 1 kHz
    pts = G["helix_pts"]
    got = np.concatenate([distance_to_helix(pts, (0.05, 0.05, 0.0), 0.04, 0.03, 2.5),
                          distance_to_helix(pts, (0.0, 0.02, 0.01), 0.02, 0.05, 0.7)])
    np.testing.assert_allclose(got, G["helix_dist"], rtol=RTOL, atol=1e-15)
    with pytest.raises(ValueError):
        distance_to_helix(pts[:, :2], (0, 0, 0), 0.1, 0.1, 1.0)
    with pytest.raises(ValueError):
        distance_to_helix(pts, (0, 0), 0.1, 0.1, 1.0)


def test_horn_flares_match_reference():
    ts = np.linspace(0, 1, 11)
    for prof in ("conical", "exponential", "hyperbolic", "tractrix"):
        h = S.Horn((0.0, 0.0, 0.05), (0.0, 0.0, 0.0), 0.006, 0.02, prof)
        want = G[f"horn_{prof}"]
        assert h.cutoff_frequency == want[0]
        np.testing.assert_array_equal(h.radius_at_position(ts), want[1:])


class _Stub:
    """The attributes a Microphone reads from its solver."""

    def __init__(self, shape, dx, dt):
        self.shape, self.dx, self.dt, self.rho, self.c = shape, dx, dt, 1.2, 343.0

    def _flush_traces(self):
        pass


def test_microphone_levels_wav_and_host_record(tmp_path):
    fs = 48000.0
    mic = S.Microphone(position=(0.0105, 0.0113, 0.0097), name="m")
    mic._initialize(_Stub((24, 24, 24), 1e-3, 1.0 / fs))
    wave_ = G["level_wave"]
    mic._data.extend(wave_.tolist())
    mic._times.extend((np.arange(wave_.size) / fs).tolist())
    for w in ("A", "C", None):
        key = w or "Z"
        assert mic.get_spl(weighting=w) == pytest.approx(
            W.calculate_spl(W.apply_weighting(wave_, fs, w).astype(np.float32)), rel=RTOL)
        assert mic.get_leq(weighting=w, duration=0.05) == pytest.approx(
            float(G[f"leq_005__{key}"][0]), rel=1e-6)
    assert mic.get_time_weighted_level(time_constant="slow").shape == wave_.shape
    path = tmp_path / "m.wav"
    mic.to_wav(str(path), sample_rate=48000, bit_depth=16)
    with wave.open(str(path), "rb") as r:
        assert (r.getnchannels(), r.getsampwidth(), r.getframerate()) == (1, 2, 48000)
        frames = np.frombuffer(r.readframes(r.getnframes()), dtype=np.int16)
    assert frames.size == wave_.size and np.abs(frames).max() == int(0.95 * 32767)
    mic.to_wav(str(path), sample_rate=24000, bit_depth=32)
    with wave.open(str(path), "rb") as r:
        assert r.getnframes() == wave_.size // 2 and r.getsampwidth() == 4
    with pytest.raises(ValueError):
        mic.to_wav(str(path), bit_depth=24)
    # one sample from host fields: the trilinear weights of the reference's
    # Python path in float32, the same sum the GPU's microphone rows form
    rng = np.random.default_rng(3)
    p = rng.standard_normal((24, 24, 24)).astype(np.float32)
    mic.clear()
    mic.record(p, 0.0)
    (_, cells, w), = mic._rows(p.shape, python_path=True)
    acc = np.float32(0.0)
    for c, wc in zip(cells, w):
        acc = np.float32(acc + np.float32(wc * p.reshape(-1)[c]))
    assert mic.get_waveform()[0] == acc
    card = S.Microphone(position=(0.0105, 0.0113, 0.0097), pattern="cardioid",
                        direction=(1.0, 0.0, 0.0))
    card._initialize(_Stub((24, 24, 24), 1e-3, 1.0 / fs))
    with pytest.raises(ValueError):
        card.record(p, 0.0)
    card.record(p, 0.0, vx=p, vy=p, vz=p)
    assert len(card.get_waveform()) == 1


def test_audio_file_waveform(tmp_path):
    """AudioFileWaveform (core/waveforms.py): integer PCM scaled to [-1, 1),
    channel mix or pick, trimming, Fourier resampling to the step rate,
    zero past the end or wrapped when looping."""
    from scipy import signal
    from scipy.io import wavfile

    sr = 8000
    left = (np.arange(400) % 50 * 600 - 15000).astype(np.int16)
    right = (-left // 2).astype(np.int16)
    path = tmp_path / "st.wav"
    wavfile.write(path, sr, np.stack([left, right], axis=1))
    mix = S.AudioFileWaveform(str(path), amplitude=2.0)
    want = np.mean(np.stack([left, right], 1).astype(np.float32) / 32768.0, axis=1)
    assert mix.num_samples == 400 and mix.native_sample_rate == sr
    assert mix.duration_seconds == pytest.approx(0.05)
    dt = 1.0 / sr  # the native rate: no resampling
    times = np.arange(402) * dt
    got = mix.waveform(times, dt)
    np.testing.assert_array_equal(got[:400], 2.0 * want.astype(np.float32))
    assert got[400] == 0 and got[401] == 0
    one = S.AudioFileWaveform(str(path), channel=1, start_time=0.01, duration=0.02, loop=True)
    assert one.num_samples == 160
    np.testing.assert_array_equal(one.waveform(np.array([0.0, 160 * dt]), dt),
                                  np.float32(right[80]) / np.float32(32768.0) * np.ones(2))
    dt2 = 1.0 / 24000
    np.testing.assert_array_equal(mix._at_rate(dt2),
                                  signal.resample(want.astype(np.float32), 1200).astype(np.float32))
    with pytest.raises(ValueError):
        S.AudioFileWaveform(str(path), channel=2)
    with pytest.raises(FileNotFoundError):
        S.AudioFileWaveform(str(tmp_path / "none.wav"))


def _pole_rows(mat):
    return np.array([[0 if p.is_debye else 1, p.delta_chi, p.tau or 0.0, p.omega_0 or 0.0,
                      p.gamma or 0.0, 0 if p.target == "density" else 1]
                     for p in mat.poles]).reshape(-1, 6)


def test_material_library_poles_match_reference():
    """Every predefined material's poles, and those of the resonant absorber
    models, equal the reference's (the porous fits run the same NumPy and
    LAPACK calls on the same inputs)."""
    from strata_fdtd_gb300 import materials as M

    names = M.list_materials()
    assert len(names) == 31 and M.list_categories()[0] == "fluids"
    for name in names:
        np.testing.assert_array_equal(_pole_rows(M.get_material(name)), G[f"lib__{name}"],
                                      err_msg=name)
    assert M.get_material("FIBERGLASS_48KG") is M.FIBERGLASS_48
    with pytest.raises(KeyError):
        M.get_material("unobtainium")
    with pytest.raises(KeyError):
        M.list_materials("metals")
    extra = {
        "helmholtz": M.HelmholtzResonator(name="h", neck_radius=0.02, neck_length=0.04,
                                          cavity_volume=0.015, loss_factor=0.12),
        "membrane": M.MembraneAbsorber(name="m", surface_density=4.2, cavity_depth=0.15),
        "perforated": M.PerforatedPanel(name="p", hole_diameter=0.003, plate_thickness=0.012,
                                        perforation_ratio=0.15, cavity_depth=0.2),
        "quarter": M.QuarterWaveResonator(name="q", length=0.858, diameter=0.1,
                                          loss_factor=0.08, n_modes=4),
        "porous_thick": M.PorousMaterial(name="pt", flow_resistivity=18000, porosity=0.97,
                                         tortuosity=1.05, viscous_length=90e-6,
                                         thermal_length=180e-6, thickness=0.05, num_poles=8),
    }
    for key, mat in extra.items():
        np.testing.assert_array_equal(_pole_rows(mat), G[f"model__{key}"], err_msg=key)
    om = 2 * np.pi * np.array([63.0, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0])
    pt = extra["porous_thick"]
    tube = M.ImpedanceTube(length=0.5, diameter=0.1, mic_spacing=0.05, sample_distance=0.1)
    resp = np.concatenate([
        pt.jca_impedance(om), pt.surface_impedance(om), pt.surface_impedance(om, backing=900.0),
        pt.absorption_coefficient_layer(om), tube.absorption_coefficient(pt, om),
        tube.absorption_coefficient(M.MDF_MEDIUM, om), M.MDF_MEDIUM.loss_factor_spectrum(om),
        M.SORBOTHANE.quality_factor(om), extra["helmholtz"].absorption_analytical(om),
        extra["perforated"].impedance_analytical(om)]).astype(complex)
    np.testing.assert_allclose(resp, G["model_resp"], rtol=1e-12)
    fit = pt.validate_pole_fit(om)
    np.testing.assert_allclose([
        extra["helmholtz"].resonance_frequency, extra["helmholtz"].quality_factor_theoretical,
        extra["membrane"].resonance_frequency, extra["perforated"].resonance_frequency,
        extra["quarter"].fundamental_frequency, M.MDF_MEDIUM.c_longitudinal,
        tube.max_frequency, tube.min_frequency, fit["density_max_error"],
        fit["modulus_mean_error"]], G["model_scalars"], rtol=1e-12)
    for bad in (dict(porosity=1.5), dict(tortuosity=0.9), dict(num_poles=1)):
        with pytest.raises(ValueError):
            M.PorousMaterial(**bad)
    with pytest.raises(ValueError):
        M.ViscoelasticSolid(poissons_ratio=0.5)


def test_loudspeaker_sources_and_regions_match_reference():
    """The cabinet builder's membrane sources (one per driver with a
    waveform: centre on its baffle face, radius, normal axis, mode) and
    absorber boxes equal the reference's (geometry/loudspeaker.py)."""
    import cases as C

    enc = C.loudspeaker_cabinet(S, waveform=S.GaussianPulse(position=(0, 0, 0), frequency=400.0))
    got = np.array([list(s.center) + [s.radius, "xyz".index(s.normal_axis), *s.mode]
                    for s in enc.get_membrane_sources()])
    np.testing.assert_array_equal(got, G["cab_sources"])
    regions = np.array([list(b.center) + list(b.size) + [mid]
                        for b, mid in enc.get_material_regions()])
    np.testing.assert_array_equal(regions, G["cab_regions"])
    with pytest.raises(ValueError):
        S.LoudspeakerEnclosure((0.2, 0.2, 0.2)).add_driver((0.1, 0.1), 0.05,
                                                           baffle_face="side").build()


def test_dsp_waveforms_match_reference():
    """Crossovers (Linkwitz-Riley, Butterworth, Bessel), a delay and
    parametric EQ bands over a pulse at 48 kHz equal the reference's
    (dsp/crossover.py, delay.py, eq.py: the same SciPy filters, biquads by
    the Audio EQ Cookbook)."""
    import cases as C

    from strata_fdtd_gb300 import dsp

    t = np.arange(1500) / 48000.0
    for key, wf in C.dsp_waveforms(S, dsp).items():
        np.testing.assert_allclose(wf.waveform(t, 1 / 48000.0), G[f"dsp__{key}"], rtol=1e-6,
                                   atol=1e-7, err_msg=key)
    with pytest.raises(ValueError):
        S.ThreeWayCrossover(low_freq=4000.0, high_freq=400.0)
    with pytest.raises(ValueError):
        S.FilteredWaveform(S.GaussianPulse(position=(0, 0, 0), frequency=1.0), "lowpass",
                           30000.0).waveform(t, 1 / 48000.0)


def test_parametric_geometry_and_constraints():
    """Parametric shapes, constraint sets and the optimiser's penalties
    (geometry/parametric.py), on the host."""
    from strata_fdtd_gb300 import geometry as G_

    h = G_.ParametricHorn(throat_radius=0.01, mouth_radius=0.04, length=0.1,
                          axis_start=(0.05, 0.05, 0.0), axis_direction=(0.0, 0.0, 2.0))
    assert [p.name for p in h.get_parameters()] == ["throat_radius", "mouth_radius", "length"]
    assert h.to_dict() == {"throat_radius": 0.01, "mouth_radius": 0.04, "length": 0.1}
    h2 = h.with_parameters(length=0.2)
    assert h2.length == 0.2 and h.length == 0.1
    horn = h2.to_sdf()
    np.testing.assert_allclose(horn.mouth_position, (0.05, 0.05, 0.2))
    p = G_.Parameter("x", 1.0, (0.0, 2.0))
    assert p.validate(1.5) and not p.validate(2.5) and p.clip(3.0) == 2.0
    cs = G_.ConstraintSet()
    cs.add_min_value("length", 0.08)
    cs.add_max_value("mouth_radius", 0.05)
    cs.add_ratio_constraint("throat_radius", "mouth_radius", 2.0)
    ok = {"length": 0.1, "mouth_radius": 0.04, "throat_radius": 0.01}
    assert cs.is_feasible(ok) and cs.total_violation(ok) == 0
    bad = {"length": 0.05, "mouth_radius": 0.06, "throat_radius": 0.04}
    v = cs.evaluate_all(bad)
    assert v["min_length"] == pytest.approx(0.03) and v["max_mouth_radius"] == pytest.approx(0.01)
    assert v["mouth_radius_over_throat_radius"] == pytest.approx(0.02)
    opt = G_.GeometryOptimizer(h, grid=S.UniformGrid((8, 8, 8), 1e-2), constraints=cs)
    assert opt.objective(np.array([0.04, 0.06, 0.05]), lambda m: 0.0) == pytest.approx(
        1e6 * (1 + 0.06))
