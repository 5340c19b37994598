"""Dispersive materials for the ADE path (materials/base.py:55-559 of
rjwalters/strata-fdtd): the pole description and its FDTD recursion
coefficients, which the time step consumes, and the material interface
around them -- high-frequency density and bulk modulus, and the
frequency-domain properties a user evaluates on the host (effective density
and modulus, wavenumber, phase and group velocity, impedance, attenuation,
reflection and absorption)."""
from __future__ import annotations

import enum
from abc import ABC, abstractmethod
from dataclasses import dataclass, field
from typing import Literal

import numpy as np


class PoleType(enum.Enum):
    DEBYE = "debye"
    LORENTZ = "lorentz"


@dataclass
class Pole:
    """One dispersion pole.  Debye: J' = alpha*J + beta*f; Lorentz:
    J' = a*J + b*J_prev + d*f (coefficients as materials/base.py:157-188)."""

    pole_type: PoleType
    delta_chi: float
    target: Literal["density", "modulus"]
    tau: float | None = None
    omega_0: float | None = None
    gamma: float | None = None

    def __post_init__(self):
        if self.pole_type == PoleType.DEBYE:
            if self.tau is None or self.tau <= 0:
                raise ValueError("Debye poles require a positive tau")
        else:
            if self.omega_0 is None or self.gamma is None:
                raise ValueError("Lorentz poles require omega_0 and gamma parameters")
            if self.omega_0 <= 0:
                raise ValueError("omega_0 must be positive")
            if self.gamma < 0:
                raise ValueError("gamma must be non-negative")
        if self.target not in ("density", "modulus"):
            raise ValueError("target must be 'density' or 'modulus'")

    @property
    def is_debye(self) -> bool:
        return self.pole_type == PoleType.DEBYE

    @property
    def is_lorentz(self) -> bool:
        return self.pole_type == PoleType.LORENTZ

    def __repr__(self) -> str:
        if self.is_debye:
            return (f"Pole(DEBYE, \u0394\u03c7={self.delta_chi:.3g}, \u03c4={self.tau:.2e}s, "
                    f"target={self.target})")
        return (f"Pole(LORENTZ, \u0394\u03c7={self.delta_chi:.3g}, "
                f"f\u2080={self.omega_0 / (2 * np.pi):.1f}Hz, \u03b3={self.gamma:.2e}, "
                f"target={self.target})")

    def susceptibility(self, omega):
        omega = np.asarray(omega)
        if self.is_debye:
            return self.delta_chi / (1 + 1j * omega * self.tau)
        return self.delta_chi * self.omega_0**2 / (self.omega_0**2 - omega**2 + 1j * self.gamma * omega)

    def fdtd_coefficients(self, dt: float) -> tuple[float, ...]:
        if self.is_debye:
            tau_dt = self.tau / dt
            denom = 1 + tau_dt
            return (tau_dt / denom, self.delta_chi / denom)
        w0, g = self.omega_0, self.gamma
        dt2 = dt * dt
        c = 1 + g * dt / 2
        a = (2 - w0**2 * dt2) / c
        b = -(1 - g * dt / 2) / c
        d = self.delta_chi * w0**2 * dt2 / c
        return (a, b, d)


class AcousticMaterial(ABC):
    """A material given by its high-frequency density rho_inf, bulk modulus
    K_inf and dispersion poles: rho(w) = rho_inf (1 + sum of the density
    poles' susceptibilities), K(w) likewise with the modulus poles
    (materials/base.py:215-507).  Subclasses supply the three."""

    name: str = "unnamed"

    @property
    @abstractmethod
    def rho_inf(self) -> float: ...

    @property
    @abstractmethod
    def K_inf(self) -> float: ...

    @property
    @abstractmethod
    def poles(self) -> list: ...

    @property
    def density_poles(self) -> list:
        return [p for p in self.poles if p.target == "density"]

    @property
    def modulus_poles(self) -> list:
        return [p for p in self.poles if p.target == "modulus"]

    @property
    def c_inf(self) -> float:
        return np.sqrt(self.K_inf / self.rho_inf)

    @property
    def Z_inf(self) -> float:
        return self.rho_inf * self.c_inf

    def _dispersed(self, base, poles, omega):
        omega = np.asarray(omega)
        total = np.ones_like(omega, dtype=complex)
        for pole in poles:
            total += pole.susceptibility(omega)
        return base * total

    def effective_density(self, omega):
        """rho(w), complex: the imaginary part is the loss."""
        return self._dispersed(self.rho_inf, self.density_poles, omega)

    def effective_modulus(self, omega):
        """K(w), complex."""
        return self._dispersed(self.K_inf, self.modulus_poles, omega)

    def wavenumber(self, omega):
        """k(w) = w sqrt(rho(w) / K(w)); Im k is the attenuation per metre."""
        omega = np.asarray(omega)
        return omega * np.sqrt(self.effective_density(omega) / self.effective_modulus(omega))

    def phase_velocity(self, omega):
        return np.real(omega / self.wavenumber(omega))

    def group_velocity(self, omega, domega: float = 1.0):
        """dw/dk by a central difference of width domega."""
        omega = np.asarray(omega)
        return domega / np.real(self.wavenumber(omega + domega / 2)
                                - self.wavenumber(omega - domega / 2))

    def impedance(self, omega):
        """Z(w) = sqrt(rho(w) K(w))."""
        omega = np.asarray(omega)
        return np.sqrt(self.effective_density(omega) * self.effective_modulus(omega))

    def attenuation(self, omega):
        """Im k(w) in Np/m."""
        return np.imag(self.wavenumber(omega))

    def attenuation_db_per_meter(self, omega):
        return 8.685889638 * self.attenuation(omega)  # 20 log10(e)

    def reflection_coefficient(self, omega, Z_other):
        Z = self.impedance(omega)
        return (Z - Z_other) / (Z + Z_other)

    def absorption_coefficient(self, omega, Z_backing):
        """1 - |R|^2 against a backing of impedance Z_backing."""
        return 1 - np.abs(self.reflection_coefficient(omega, Z_backing)) ** 2

    def n_poles(self) -> int:
        return len(self.poles)

    def n_density_poles(self) -> int:
        return len(self.density_poles)

    def n_modulus_poles(self) -> int:
        return len(self.modulus_poles)

    def summary(self) -> str:
        lines = [f"Material: {self.name}",
                 f"  \u03c1\u221e = {self.rho_inf:.2f} kg/m\u00b3",
                 f"  K\u221e = {self.K_inf:.2e} Pa",
                 f"  c\u221e = {self.c_inf:.1f} m/s",
                 f"  Z\u221e = {self.Z_inf:.1f} Pa\u00b7s/m",
                 f"  Poles: {self.n_poles()} ({self.n_density_poles()} density, "
                 f"{self.n_modulus_poles()} modulus)"]
        lines += [f"    [{q}] {pole}" for q, pole in enumerate(self.poles)]
        return "\n".join(lines)


Material = AcousticMaterial


@dataclass
class SimpleMaterial(AcousticMaterial):
    """Constant rho and c, plus optional poles (materials/base.py:509-555)."""

    name: str = "material"
    _rho: float = field(default=1.2, repr=False)
    _c: float = field(default=343.0, repr=False)
    _poles: list = field(default_factory=list, repr=False)

    @property
    def rho_inf(self) -> float:
        return self._rho

    @property
    def K_inf(self) -> float:
        return self._rho * self._c**2

    @property
    def poles(self) -> list:
        return self._poles

    @classmethod
    def from_impedance(cls, name: str, rho: float, Z: float) -> "SimpleMaterial":
        """The material of density rho and characteristic impedance Z."""
        return cls(name=name, _rho=rho, _c=Z / rho)


AIR_20C = SimpleMaterial(name="air_20C", _rho=1.204, _c=343.0)

# the material models and the predefined library, under this module's name
# as under the reference's materials package
from .material_models import (  # noqa: E402
    DampingMaterial, HelmholtzResonator, ImpedanceTube, MembraneAbsorber, PerforatedPanel,
    PorousMaterial, QuarterWaveResonator, ViscoelasticSolid)
from .material_library import (  # noqa: E402
    ACOUSTIC_FOAM_DENSE, ACOUSTIC_FOAM_OPEN, AIR_15C, AIR_25C, BUTYL_RUBBER, COTTON_BATTING,
    EPDM_RUBBER, FIBERGLASS_24, FIBERGLASS_32, FIBERGLASS_48, FIBERGLASS_96, HARDWOOD_OAK,
    MATERIALS, MDF_HIGH, MDF_LIGHT, MDF_MEDIUM, MINERAL_WOOL_40, MINERAL_WOOL_60,
    MINERAL_WOOL_100, NEOPRENE, OSB, PARTICLE_BOARD, PLYWOOD_BIRCH, PLYWOOD_MARINE,
    PLYWOOD_SOFTWOOD, POLYESTER_BATTING, POLYURETHANE_FOAM, SILICONE_RUBBER, SORBOTHANE,
    WATER_20C, WOOL_FELT, get_material, list_categories, list_materials, material_summary)
