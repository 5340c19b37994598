"""Loudspeaker cabinets as SDF geometry (geometry/loudspeaker.py of
rjwalters/strata-fdtd).

``LoudspeakerEnclosure`` assembles a cabinet from the voxeliser's shapes: a
box shell of ``wall_thickness``, horizontal chamber dividers (with holes),
braces, driver cutouts and reflex ports (cylinders, or cones when flared)
through a baffle face, and Helmholtz resonator arrays cut into the solid;
absorber regions become material boxes and drivers with a waveform become
circular membrane sources.  The construction follows the reference's
arithmetic, so the voxelised cabinet is the reference's mask.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .resonator import helmholtz_array
from .sdf import Box, Cone, Cylinder, Difference, Union

_NORMAL = {"front": "y", "back": "y", "left": "x", "right": "x", "top": "z", "bottom": "z"}


@dataclass
class LoudspeakerEnclosure:
    """Cabinet of ``external_size`` (width x, depth y, height z, metres)
    with walls of ``wall_thickness``; the front baffle is the y = 0 face.
    The ``add_*`` methods return the enclosure for chaining; ``build``
    returns the solid."""

    external_size: tuple
    wall_thickness: float = 0.019
    _drivers: list = field(default_factory=list, init=False, repr=False)
    _ports: list = field(default_factory=list, init=False, repr=False)
    _chambers: list = field(default_factory=list, init=False, repr=False)
    _bracing: list = field(default_factory=list, init=False, repr=False)
    _absorbers: list = field(default_factory=list, init=False, repr=False)
    _resonators: list = field(default_factory=list, init=False, repr=False)

    def __post_init__(self):
        centre = tuple(np.array(self.external_size) / 2)
        inner = Box(center=centre,
                    size=tuple(s - 2 * self.wall_thickness for s in self.external_size))
        self._shell = Difference(Box(center=centre, size=self.external_size), inner)
        self._cavity = inner  # the air inside

    # -- description ---------------------------------------------------------
    def add_driver(self, position, diameter, mounting_depth=0.0, baffle_face="front",
                   name=None, waveform=None, mode=(0, 1)):
        """A driver cutout of ``diameter`` at ``position`` on a baffle face;
        with a waveform it is also a membrane source (mode (m, n))."""
        self._drivers.append(dict(position=position, diameter=diameter, depth=mounting_depth,
                                  face=baffle_face, name=name or f"driver_{len(self._drivers)}",
                                  waveform=waveform, mode=mode))
        return self

    def add_port(self, position, diameter, length, baffle_face="front", flare_ratio=1.0,
                 flare_length=0.0):
        """A reflex port tube of ``length`` from a baffle face inward, a cone
        widening to ``flare_ratio`` times the diameter at the mouth when
        flared."""
        self._ports.append(dict(position=position, diameter=diameter, length=length,
                                face=baffle_face, flare_ratio=flare_ratio,
                                flare_length=flare_length))
        return self

    def add_chamber_divider(self, z_position, thickness=0.019, hole_positions=None):
        """A horizontal divider at height z, with (x, y, diameter) holes."""
        self._chambers.append(dict(z=z_position, thickness=thickness,
                                   holes=hole_positions or []))
        return self

    def add_brace(self, start, end, width, height):
        """A brace beam of width x height centred between start and end,
        its length along z."""
        self._bracing.append(dict(start=start, end=end, width=width, height=height))
        return self

    def add_absorber_region(self, bounds, material_id=1):
        """A box of absorbing material between two corners."""
        self._absorbers.append(dict(bounds=bounds, material_id=material_id))
        return self

    def add_helmholtz_array(self, region_bounds, frequency_range, n_resonators):
        """Resonators log-spaced over the frequency range, laid out in the
        region (10 mm necks of 3 mm radius, box cavities), cut from the solid."""
        self._resonators.append(dict(bounds=region_bounds, freq_range=frequency_range,
                                     n=n_resonators))
        return self

    # -- products ------------------------------------------------------------
    def build(self):
        """The cabinet solid: shell, dividers and braces, minus divider holes,
        driver cutouts and ports, minus each resonator in turn."""
        parts, cuts = [self._shell], []
        for ch in self._chambers:
            parts.append(self._divider(ch))
            cuts += [self._divider_hole(x, y, ch["z"], ch["thickness"], d)
                     for x, y, d in ch["holes"]]
        parts += [self._brace(b) for b in self._bracing]
        solid = Union(*parts) if len(parts) > 1 else parts[0]
        cuts += [self._driver_cutout(d) for d in self._drivers]
        cuts += [self._port(p) for p in self._ports]
        if cuts:
            solid = Difference(solid, *cuts)
        for spec in self._resonators:
            for r in self._helmholtz(spec):
                solid = Difference(solid, r)
        return solid

    def get_material_regions(self):
        """[(box, material id)] of the absorber regions."""
        out = []
        for a in self._absorbers:
            lo, hi = a["bounds"]
            out.append((Box(center=tuple(np.mean([lo, hi], axis=0)),
                            size=tuple(np.abs(np.array(hi) - np.array(lo)))), a["material_id"]))
        return out

    def get_membrane_sources(self):
        """A circular membrane source per driver given a waveform."""
        from .membranes import CircularMembraneSource

        return [CircularMembraneSource(center=self._driver_position_to_3d(d),
                                       radius=d["diameter"] / 2,
                                       normal_axis=self._face_to_normal_axis(d["face"]),
                                       waveform=d["waveform"], mode=d["mode"])
                for d in self._drivers if d["waveform"] is not None]

    # -- pieces ----------------------------------------------------------------
    def _driver_position_to_3d(self, driver):
        (a, b), face = driver["position"], driver["face"]
        w, d, h = self.external_size
        where = {"front": (a, 0.0, b), "back": (a, d, b), "top": (a, b, h),
                 "bottom": (a, b, 0.0), "left": (0.0, a, b), "right": (w, a, b)}
        if face not in where:
            raise ValueError(f"Unknown face: {face}")
        return where[face]

    def _face_to_normal_axis(self, face):
        if face not in _NORMAL:
            raise ValueError(f"Unknown face: {face}")
        return _NORMAL[face]

    def _helmholtz(self, spec):
        lo, hi = spec["bounds"]
        region = Box(center=tuple(np.mean([lo, hi], axis=0)),
                     size=tuple(np.abs(np.array(hi) - np.array(lo))))
        return helmholtz_array(region=region, frequency_range=spec["freq_range"],
                               n_resonators=spec["n"], spacing="log", cavity_shape="box",
                               neck_length=0.01, neck_radius=0.003)

    def _divider(self, ch):
        w, d, _ = self.external_size
        t2 = 2 * self.wall_thickness
        return Box(center=(w / 2, d / 2, ch["z"]), size=(w - t2, d - t2, ch["thickness"]))

    @staticmethod
    def _divider_hole(x, y, z, thickness, diameter):
        return Cylinder(p1=(x, y, z - thickness / 2 - 0.001), p2=(x, y, z + thickness / 2 + 0.001),
                        radius=diameter / 2)

    @staticmethod
    def _brace(brace):
        start, end = np.array(brace["start"]), np.array(brace["end"])
        return Box(center=tuple((start + end) / 2),
                   size=(brace["width"], brace["height"], np.linalg.norm(end - start)))

    def _driver_cutout(self, driver):
        """A cylinder from just outside the baffle to the mounting depth --
        the reference's end points per face (loudspeaker.py:560-603)."""
        pos, depth, face = driver["position"], driver["depth"], driver["face"]
        w, d, h = self.external_size
        a, b = pos
        ends = {"front": ((a, -0.001, b), (a, depth, b)),
                "back": ((a, 0, b), (a, d + 0.001, b)),
                "top": ((a, b, 0), (a, b, h + 0.001)),
                "bottom": ((a, b, -0.001), (a, b, h)),
                "left": ((-0.001, a, b), (w, a, b)),
                "right": ((0, a, b), (w + 0.001, a, b))}
        if face not in ends:
            raise ValueError(f"Unknown baffle face: {face}")
        p1, p2 = ends[face]
        return Cylinder(p1=p1, p2=p2, radius=driver["diameter"] / 2)

    def _port(self, port):
        """The port from its mouth just outside the face to its throat
        ``length`` inside (loudspeaker.py:605-654)."""
        pos, L, face = port["position"], port["length"], port["face"]
        w, d, h = self.external_size
        a, b = pos
        ends = {"front": ((a, -0.001, b), (a, L, b)),
                "back": ((a, d + 0.001, b), (a, d - L, b)),
                "top": ((a, b, h + 0.001), (a, b, h - L)),
                "bottom": ((a, b, -0.001), (a, b, L)),
                "left": ((-0.001, a, b), (L, a, b)),
                "right": ((w + 0.001, a, b), (w - L, a, b))}
        if face not in ends:
            raise ValueError(f"Unknown baffle face: {face}")
        p1, p2 = ends[face]
        r = port["diameter"] / 2
        if port["flare_ratio"] > 1.0 and port["flare_length"] > 0:
            return Cone(p1=p1, p2=p2, r1=port["diameter"] / 2 * port["flare_ratio"], r2=r)
        return Cylinder(p1=p1, p2=p2, radius=r)


def tower_speaker(width, depth, height, woofer_diameter, midrange_diameter, tweeter_diameter):
    """Three-way tower: tweeter, midrange and woofer on the front baffle at
    85, 60 and 25 % of the height, dividers at 45 and 75 %."""
    enc = LoudspeakerEnclosure(external_size=(width, depth, height))
    cx = width / 2
    enc.add_driver((cx, height * 0.85), tweeter_diameter, baffle_face="front", name="tweeter")
    enc.add_driver((cx, height * 0.6), midrange_diameter, baffle_face="front", name="midrange")
    enc.add_driver((cx, height * 0.25), woofer_diameter, baffle_face="front", name="woofer")
    enc.add_chamber_divider(z_position=height * 0.45)
    enc.add_chamber_divider(z_position=height * 0.75)
    return enc


def bookshelf_speaker(width, depth, height, woofer_diameter, tweeter_diameter,
                      port_diameter=0.05, port_length=0.15):
    """Two-way bookshelf: tweeter and woofer on the front baffle at 75 and
    35 % of the height, a rear reflex port at 15 %."""
    enc = LoudspeakerEnclosure(external_size=(width, depth, height))
    cx = width / 2
    enc.add_driver((cx, height * 0.75), tweeter_diameter, baffle_face="front", name="tweeter")
    enc.add_driver((cx, height * 0.35), woofer_diameter, baffle_face="front", name="woofer")
    enc.add_port((cx, height * 0.15), port_diameter, port_length, baffle_face="back")
    return enc
