"""Error behaviour of the drop-in API: the invalid inputs the reference's own
tests reject (tests/test_sdf.py, test_sdf_csg.py, test_transformations.py,
test_paths.py, test_grid.py, test_resonator.py, test_dsp.py,
test_weighting.py, test_waveforms.py, test_loudspeaker.py,
test_materials.py, test_microphone*.py, test_*membrane*.py,
test_material_geometry.py of rjwalters/strata-fdtd) raise the same
exception type here, with a message that matches the same pattern.  Only
objects that need no GPU are built."""
import numpy as np
import pytest

import strata_fdtd_gb300 as S
from strata_fdtd_gb300 import materials as M
from strata_fdtd_gb300.geometry import (HelixPath, LoudspeakerEnclosure, MaterializedGeometry,
                                        MaterialVolume, SpiralPath)
from strata_fdtd_gb300.weighting import get_weighting_sos

BOX = S.Box(center=(0, 0, 0), size=(0.02, 0.02, 0.02))
SPH = S.Sphere(center=(0, 0, 0), radius=1.0)
WF = S.GaussianPulse(position=(0, 0, 0), frequency=200.0)
SPIRAL = dict(center=(0.15, 0.15), throat_radius=0.025, mouth_radius=0.075,
              inner_spiral_radius=0.04, outer_spiral_radius=0.12, turns=2.5, height=0.15)
HELIX = dict(center=(0.1, 0.1, 0.0), helix_radius=0.06, tube_radius_start=0.02,
             tube_radius_end=0.02, pitch=0.04, turns=3.0)
HORN = dict(throat_position=(0, 0, 0.1), mouth_position=(0, 0, 0), throat_radius=0.01,
            mouth_radius=0.02, profile="conical")
RES = dict(position=(0.05, 0.05, 0.05), cavity_shape="box", cavity_size=(0.03, 0.03, 0.03),
           neck_length=0.01, neck_radius=0.005)
CIRC = dict(center=(0.05, 0.05, 0.05), radius=0.02, normal_axis="z", waveform=WF)
RECT = dict(center=(0.05, 0.05, 0.05), size=(0.04, 0.04), normal_axis="z", waveform=WF)
ENC = LoudspeakerEnclosure(external_size=(0.2, 0.25, 0.4))
MIC = (0.05, 0.05, 0.05)

CASES = [
    # SDF primitives and CSG
    ("box_missing_size", lambda: S.Box(center=(0, 0, 0)), ValueError, "Must provide either"),
    ("box_missing_corner", lambda: S.Box(min_corner=(0, 0, 0)), ValueError, "Must provide either"),
    ("box_negative", lambda: S.Box(center=(0, 0, 0), size=(-1, 1, 1)), ValueError,
     "must be positive"),
    ("sphere_negative", lambda: S.Sphere(center=(0, 0, 0), radius=-1), ValueError,
     "must be positive"),
    ("cylinder_negative", lambda: S.Cylinder(p1=(0, 0, 0), p2=(0, 0, 1), radius=-1), ValueError,
     "must be positive"),
    ("cylinder_coincident", lambda: S.Cylinder(p1=(0, 0, 0), p2=(0, 0, 0), radius=0.01),
     ValueError, "must be distinct"),
    ("cone_negative", lambda: S.Cone(p1=(0, 0, 0), p2=(0, 0, 1), r1=-1, r2=0.5), ValueError,
     "must be non-negative"),
    ("cone_zero_radii", lambda: S.Cone(p1=(0, 0, 0), p2=(0, 0, 1), r1=0, r2=0), ValueError,
     "cannot have both radii zero"),
    ("cone_coincident", lambda: S.Cone(p1=(0, 0, 0), p2=(0, 0, 0), r1=1, r2=0.5), ValueError,
     "must be distinct"),
    ("spiral_radii", lambda: S.SpiralHorn(**{**SPIRAL, "throat_radius": -0.01}), ValueError,
     "radii must be positive"),
    ("spiral_height", lambda: S.SpiralHorn(**{**SPIRAL, "height": 0.0}), ValueError,
     "Height must be positive"),
    ("spiral_profile", lambda: S.SpiralHorn(**SPIRAL, profile="invalid"), ValueError,
     "profile must be"),
    ("helix_radius", lambda: S.HelicalTube(**{**HELIX, "helix_radius": 0.0}), ValueError,
     "helix_radius must be positive"),
    ("helix_tube", lambda: S.HelicalTube(**{**HELIX, "tube_radius_start": -0.01}), ValueError,
     "tube radii must be positive"),
    ("helix_pitch", lambda: S.HelicalTube(**{**HELIX, "pitch": 0.0}), ValueError,
     "pitch must be positive"),
    ("horn_profile", lambda: S.Horn(**{**HORN, "profile": "invalid"}), ValueError,
     "profile must be one of"),
    ("horn_throat", lambda: S.Horn(**{**HORN, "throat_radius": -0.01}), ValueError,
     "must be positive"),
    ("horn_mouth", lambda: S.Horn(**{**HORN, "mouth_radius": 0}), ValueError, "must be positive"),
    ("horn_coincident", lambda: S.Horn(**{**HORN, "throat_position": (0, 0, 0)}), ValueError,
     "must be distinct"),
    ("smooth_zero", lambda: S.SmoothUnion(SPH, SPH, radius=0.0), ValueError,
     "radius must be positive"),
    ("smooth_negative", lambda: S.SmoothUnion(SPH, SPH, radius=-0.5), ValueError,
     "radius must be positive"),
    # transformations
    ("translate_2", lambda: S.Translate(BOX, [1, 2]), ValueError, "must be a 3-element vector"),
    ("translate_4", lambda: S.Translate(BOX, [1, 2, 3, 4]), ValueError,
     "must be a 3-element vector"),
    ("scale_negative", lambda: S.Scale(BOX, scale=-1.0), ValueError, "must be positive"),
    ("scale_axis", lambda: S.Scale(BOX, scale=(1.0, -1.0, 1.0)), ValueError, "must be positive"),
    ("scale_zero", lambda: S.Scale(BOX, scale=0.0), ValueError, "must be positive"),
    ("scale_method", lambda: BOX.scale((-1, 1, 1)), ValueError, "must be positive"),
    ("rotate_nothing", lambda: S.Rotate(BOX), ValueError, "Must provide either"),
    ("rotate_no_angle", lambda: S.Rotate(BOX, axis=(0, 0, 1)), ValueError, "Must provide either"),
    ("rotate_no_axis", lambda: S.Rotate(BOX, angle=np.pi / 2), ValueError, "Must provide either"),
    ("rotate_2x2", lambda: S.Rotate(BOX, matrix=np.eye(2)), ValueError, "must be 3x3"),
    ("rotate_4x4", lambda: S.Rotate(BOX, matrix=np.eye(4)), ValueError, "must be 3x3"),
    # paths
    ("spiral_inner", lambda: SpiralPath(center=(0.1, 0.1), inner_radius=0.0, outer_radius=0.1,
                                        turns=2.0), ValueError, "inner_radius must be positive"),
    ("spiral_outer", lambda: SpiralPath(center=(0.1, 0.1), inner_radius=0.1, outer_radius=0.05,
                                        turns=2.0), ValueError, "outer_radius.*must be >"),
    ("spiral_turns", lambda: SpiralPath(center=(0.1, 0.1), inner_radius=0.04, outer_radius=0.08,
                                        turns=0.0), ValueError, "turns must be positive"),
    ("spiral_type", lambda: SpiralPath(center=(0.1, 0.1), inner_radius=0.04, outer_radius=0.08,
                                       turns=2.0, spiral_type="invalid"), ValueError,
     "spiral_type must be"),
    ("helixpath_radius", lambda: HelixPath(center=(0.1, 0.1, 0.0), radius=-0.05, pitch=0.04,
                                           turns=3.0), ValueError, "radius must be positive"),
    ("helixpath_pitch", lambda: HelixPath(center=(0.1, 0.1, 0.0), radius=0.06, pitch=0.0,
                                          turns=3.0), ValueError, "pitch must be positive"),
    # grids
    ("grid_contiguous", lambda: S.NonuniformGrid.from_regions(
        x_regions=[(0.0, 0.01, 1e-3), (0.02, 0.03, 1e-3)]), ValueError, "contiguous"),
    ("grid_monotonic", lambda: S.NonuniformGrid(x_coords=np.array([0, 0.02, 0.01, 0.03]),
                                                y_coords=np.arange(4.0),
                                                z_coords=np.arange(4.0)), ValueError,
     "monotonically increasing"),
    ("grid_one_point", lambda: S.NonuniformGrid(x_coords=np.array([0.05]),
                                                y_coords=np.arange(4.0),
                                                z_coords=np.arange(4.0)), ValueError,
     "at least 2"),
    # Helmholtz resonators
    ("res_shape", lambda: S.HelmholtzResonator(**{**RES, "cavity_shape": "triangle"}),
     ValueError, "Unknown cavity_shape"),
    ("res_direction", lambda: S.HelmholtzResonator(**RES, neck_direction=(0, 0, 0)), ValueError,
     "cannot be zero"),
    ("res_neck_length", lambda: S.HelmholtzResonator(**{**RES, "neck_length": -0.01}),
     ValueError, "must be positive"),
    ("res_neck_radius", lambda: S.HelmholtzResonator(**{**RES, "neck_radius": -0.005}),
     ValueError, "must be positive"),
    ("res_box_size", lambda: S.HelmholtzResonator(**{**RES, "cavity_size": (0.03, 0.03)}),
     ValueError, "requires 3 size parameters"),
    ("res_sphere_size", lambda: S.HelmholtzResonator(**{**RES, "cavity_shape": "sphere",
                                                         "cavity_size": (0.03, 0.03)}),
     ValueError, "requires 1 size parameter"),
    ("array_range", lambda: S.helmholtz_array(region=BOX, frequency_range=(1000, 500),
                                              n_resonators=4), ValueError,
     "Invalid frequency range"),
    ("array_spacing", lambda: S.helmholtz_array(region=BOX, frequency_range=(400, 800),
                                                n_resonators=4, spacing="exponential"),
     ValueError, "spacing must be"),
    # signal processing and levels
    ("crossover_order", lambda: S.ThreeWayCrossover(low_freq=4000, high_freq=500), ValueError,
     "low_freq.*must be less than"),
    ("crossover_equal", lambda: S.ThreeWayCrossover(low_freq=2000, high_freq=2000), ValueError,
     "low_freq.*must be less than"),
    ("weighting", lambda: get_weighting_sos("X", 48000.0), ValueError, "Unknown weighting"),
    ("audio_missing", lambda: S.AudioFileWaveform("/nonexistent/path/audio.wav"),
     FileNotFoundError, "Audio file not found"),
    # cabinets
    ("face_axis", lambda: ENC._face_to_normal_axis("invalid"), ValueError, "Unknown face"),
    ("face_position", lambda: ENC._driver_position_to_3d(dict(position=(0.1, 0.2),
                                                               face="invalid")),
     ValueError, "Unknown face"),
    # materials
    ("pole_tau", lambda: S.Pole(pole_type=S.PoleType.DEBYE, delta_chi=0.5, target="modulus"),
     ValueError, "tau"),
    ("pole_omega", lambda: S.Pole(pole_type=S.PoleType.LORENTZ, delta_chi=0.5,
                                  target="modulus"), ValueError, "omega_0"),
    ("pole_target", lambda: S.Pole(pole_type=S.PoleType.DEBYE, delta_chi=0.5, tau=1e-5,
                                   target="invalid"), ValueError, "target"),
    ("porous_flow", lambda: M.PorousMaterial(flow_resistivity=-1000), ValueError,
     "flow_resistivity"),
    ("porous_porosity", lambda: M.PorousMaterial(porosity=1.5), ValueError, "porosity"),
    ("porous_tortuosity", lambda: M.PorousMaterial(tortuosity=0.5), ValueError, "tortuosity"),
    ("porous_thickness", lambda: M.PorousMaterial(flow_resistivity=10000).surface_impedance(
        2 * np.pi * 1000), ValueError, "thickness"),
    ("library_missing", lambda: M.get_material("nonexistent_material"), KeyError, None),
    ("volume_corners", lambda: MaterialVolume.from_corners(
        min_corner=(0.1, 0.1, 0.1), max_corner=(0.0, 0.0, 0.0), material=M.FIBERGLASS_48),
     ValueError, "min_corner must be less than max_corner"),
    # microphones
    ("mic_pattern", lambda: S.Microphone(position=MIC, pattern="invalid"), ValueError,
     "Unknown pattern"),
    ("mic_pattern_type", lambda: S.Microphone(position=MIC, pattern=42), TypeError,
     "must be str or callable"),
    ("mic_direction", lambda: S.Microphone(position=MIC, direction=(0, 0, 0)), ValueError,
     "direction vector cannot be zero"),
    ("mic_up", lambda: S.Microphone(position=MIC, up=(0, 0, 0)), ValueError,
     "up vector cannot be zero"),
    ("mic_parallel", lambda: S.Microphone(position=MIC, direction=(0, 0, 1), up=(0, 0, 1)),
     ValueError, "cannot be parallel"),
    ("mic_rate", lambda: S.Microphone(position=MIC).get_sample_rate(), RuntimeError,
     "not initialized"),
    ("mic_record", lambda: S.Microphone(position=MIC).record(np.zeros((10, 10, 10)), 0.0),
     RuntimeError, "not initialized"),
    # membrane sources
    ("circ_m", lambda: S.CircularMembraneSource(**CIRC, mode=(-1, 1)), ValueError,
     "Azimuthal mode m must be non-negative"),
    ("circ_n0", lambda: S.CircularMembraneSource(**CIRC, mode=(0, 0)), ValueError,
     "Radial mode n must be positive"),
    ("circ_nneg", lambda: S.CircularMembraneSource(**CIRC, mode=(0, -1)), ValueError,
     "Radial mode n must be positive"),
    ("rect_m", lambda: S.RectangularMembraneSource(**RECT, mode=(0, 1)), ValueError,
     "Mode index m must be >= 1"),
    ("rect_n", lambda: S.RectangularMembraneSource(**RECT, mode=(1, 0)), ValueError,
     "Mode index n must be >= 1"),
    ("rect_mneg", lambda: S.RectangularMembraneSource(**RECT, mode=(-1, 1)), ValueError,
     "Mode index m must be >= 1"),
]


@pytest.mark.parametrize("name,make,exc,pattern", CASES, ids=[c[0] for c in CASES])
def test_rejects_like_the_reference(name, make, exc, pattern):
    with pytest.raises(exc, match=pattern):
        make()


def test_audio_channel_and_start_time(tmp_path):
    from scipy.io import wavfile

    path = tmp_path / "st.wav"
    wavfile.write(path, 8000, np.zeros((800, 2), dtype=np.int16))
    with pytest.raises(ValueError, match="Channel 5 requested but file only has 2 channels"):
        S.AudioFileWaveform(path, channel=5)
    with pytest.raises(ValueError, match="start_time.*is beyond end of file"):
        S.AudioFileWaveform(path, start_time=1.0)


def test_membrane_base_class_and_region_cap():
    grid = S.UniformGrid(shape=(10, 10, 10), resolution=1e-2)
    base = S.MembraneSource(center=(0.05, 0.05, 0.05), normal_axis="z", waveform=WF)
    with pytest.raises(NotImplementedError, match="Subclasses must implement mode_shape"):
        base.mode_shape(np.zeros(3), np.zeros(3))
    with pytest.raises(NotImplementedError, match="Subclasses must implement get_injection_mask"):
        base.get_injection_mask(grid)
    with pytest.raises(NotImplementedError,
                       match="Subclasses must implement get_injection_weights"):
        base.get_injection_weights(grid)
    geo = MaterializedGeometry(S.Box(center=(0.05, 0.05, 0.05), size=(0.1, 0.1, 0.1)))
    for _ in range(255):
        geo.set_material(S.Sphere(center=(0.05, 0.05, 0.05), radius=0.01), M.FIBERGLASS_48)
    with pytest.raises(ValueError, match="Maximum of 255 material regions exceeded"):
        geo.set_material(S.Sphere(center=(0.05, 0.05, 0.05), radius=0.01), M.FIBERGLASS_48)


def test_microphone_without_data():
    class _Stub:
        shape, dx, dt, rho, c = (10, 10, 10), 1e-2, 1e-5, 1.2, 343.0

        def _flush_traces(self):
            pass

    mic = S.Microphone(position=MIC)
    mic._initialize(_Stub())
    for call in (mic.get_spl, mic.get_leq, mic.get_time_weighted_level,
                 lambda: mic.to_wav("x.wav")):
        with pytest.raises(RuntimeError, match="No data recorded"):
            call()
