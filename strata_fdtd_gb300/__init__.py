"""strata_fdtd_gb300 -- the strata-fdtd time-step path on GB300 (sm_103a).

A drop-in for ``FDTDSolver(backend="native")`` of rjwalters/strata-fdtd:
same classes and arguments, with the per-step stencil, rigid walls, PML, ADE
materials, sources, probes, microphones and SDF voxelisation running as
hand-written CUDA kernels behind a C ABI (include/sf_gb300.h) loaded with
ctypes.  ``BatchedSolver`` steps many solvers in one persistent launch,
``server.SolveServer`` serves a stream of solves with continuous batching,
and ``DifferentiableSolver`` differentiates a probe loss with respect to a
per-cell density field by a reverse-time adjoint.
"""
from ._native import NativeError, build
from .adjoint import DifferentiableSolver
from .batch import BatchedSolver
from .boundaries import PML, ABCFirstOrder, RadiationImpedance, RigidBoundary
from .dsp import (Crossover, DelayedWaveform, FilteredWaveform, ParametricEQ,
                  ThreeWayCrossover)
from .grid import NonuniformGrid, UniformGrid
from .loudspeaker import LoudspeakerEnclosure, bookshelf_speaker, tower_speaker
from .material_assignment import MaterializedGeometry, MaterialVolume
from .microphones import POLAR_PATTERNS, Microphone
from .materials import AIR_20C, AcousticMaterial, Material, Pole, PoleType, SimpleMaterial
from .membranes import CircularMembraneSource, MembraneSource, RectangularMembraneSource
from .resonator import HelmholtzResonator, helmholtz_array
from .paths import HelixPath, SpiralPath, distance_to_polyline
from .sdf import (Box, Cone, CSGNode, Cylinder, Difference, HelicalTube, Horn, Intersection,
                  Rotate, Scale, SDFPrimitive, SmoothDifference, SmoothIntersection, SmoothUnion,
                  Sphere, SpiralHorn, Translate, Union, conical_horn, exponential_horn,
                  hyperbolic_horn, rotation_matrix, tractrix_horn)
from .solver import (FDTDSolver, GaussianPulse, Probe, get_native_info, has_gpu_backend,
                     has_native_kernels)
from .waveforms import AudioFileWaveform
from .weighting import apply_weighting, calculate_leq, calculate_spl

from . import analysis, dsp, geometry, io, materials  # noqa: E402  (submodules by name)

__version__ = "0.1.0"

__all__ = [
    "FDTDSolver", "GaussianPulse", "AudioFileWaveform", "Probe", "POLAR_PATTERNS",
    "apply_weighting", "calculate_spl", "calculate_leq", "Crossover", "ThreeWayCrossover",
    "FilteredWaveform", "DelayedWaveform", "ParametricEQ", "Microphone", "UniformGrid", "NonuniformGrid", "PML",
    "RigidBoundary", "ABCFirstOrder", "RadiationImpedance", "Pole",
    "PoleType", "SimpleMaterial", "AcousticMaterial", "Material", "AIR_20C", "SDFPrimitive", "CSGNode", "Box", "Sphere",
    "Cylinder", "Union", "Intersection", "Difference", "Translate", "Scale", "Rotate",
    "LoudspeakerEnclosure", "bookshelf_speaker", "tower_speaker",
    "rotation_matrix", "Cone", "Horn", "SpiralHorn", "HelicalTube", "SmoothUnion",
    "SmoothIntersection", "SmoothDifference", "conical_horn", "exponential_horn",
    "hyperbolic_horn", "tractrix_horn", "SpiralPath", "HelixPath", "distance_to_polyline",
    "HelmholtzResonator", "helmholtz_array", "has_native_kernels", "has_gpu_backend", "get_native_info", "build",
    "NativeError", "BatchedSolver", "DifferentiableSolver", "MembraneSource",
    "CircularMembraneSource", "RectangularMembraneSource", "MaterializedGeometry",
    "MaterialVolume",
]
