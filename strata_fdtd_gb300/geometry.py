"""The geometry names under one module, as the reference's geometry package
groups them (geometry/__init__.py of rjwalters/strata-fdtd): SDF shapes and
CSG, paths, Helmholtz resonators, loudspeaker cabinets and material
assignment."""
from .loudspeaker import LoudspeakerEnclosure, bookshelf_speaker, tower_speaker  # noqa: F401
from .material_assignment import MaterializedGeometry, MaterialVolume  # noqa: F401
from .parametric import (ConstraintSet, GeometricConstraint, GeometryOptimizer,  # noqa: F401
                         Parameter, ParametricHorn, ParametricPrimitive)
from .paths import HelixPath, SpiralPath, distance_to_helix, distance_to_polyline  # noqa: F401
from .resonator import HelmholtzResonator, helmholtz_array  # noqa: F401
from .sdf import (Box, Cone, CSGNode, Cylinder, Difference, HelicalTube, Horn,  # noqa: F401
                  Intersection, Rotate, Scale, SDFPrimitive, SmoothDifference,
                  SmoothIntersection, SmoothUnion, Sphere, SpiralHorn, Translate, Union,
                  conical_horn, exponential_horn, hyperbolic_horn, rotation_matrix,
                  tractrix_horn)
