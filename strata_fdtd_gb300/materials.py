"""Dispersive materials for the ADE path (materials/base.py:55-213, 509-545
of rjwalters/strata-fdtd).  Only the pieces the time step consumes: the pole
description, its FDTD recursion coefficients and the high-frequency
density / bulk modulus of a material."""
from __future__ import annotations

import enum
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


@dataclass
class SimpleMaterial:
    """Constant rho and c, plus optional poles (materials/base.py:509-545)."""

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
    def c_inf(self) -> float:
        return self._c

    @property
    def poles(self) -> list:
        return self._poles

    def n_poles(self) -> int:
        return len(self._poles)


AIR_20C = SimpleMaterial(name="air_20C", _rho=1.204, _c=343.0)
