"""Material models that reduce to dispersion poles (materials/porous.py,
solids.py and resonators.py of rjwalters/strata-fdtd).

Each model computes its Debye or Lorentz poles on the host with the
reference's NumPy arithmetic; the solver's ADE path then steps them like any
other material.  The pole fits of porous materials use a least-squares solve
(LAPACK), so their last bits follow the machine's LAPACK build.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from math import pi

import numpy as np

from .materials import AcousticMaterial, Pole, PoleType

AIR_DENSITY = 1.204      # kg/m^3
AIR_VISCOSITY = 1.81e-5  # Pa s
AIR_PRANDTL = 0.71
AIR_GAMMA = 1.4
AIR_PRESSURE = 101325    # Pa
AIR_SPEED = 343.0        # m/s


def _debye_fit(tau, omega, target):
    """Real pole strengths d_j minimising |sum_j d_j / (1 + i w tau_j) -
    (target - 1)| over the sample frequencies, real and imaginary parts
    stacked (porous.py:206-280)."""
    basis = np.zeros((len(omega), len(tau)), dtype=complex)
    for j, t in enumerate(tau):
        basis[:, j] = 1 / (1 + 1j * omega * t)
    a = np.vstack([np.real(basis), np.imag(basis)])
    b = np.concatenate([np.real(target) - 1, np.imag(target)])
    return np.linalg.lstsq(a, b, rcond=None)[0]


@dataclass
class PorousMaterial(AcousticMaterial):
    """Fibrous or foam absorber by the Johnson-Champoux-Allard model
    (porous.py:32-493): flow resistivity sigma, porosity phi, tortuosity
    alpha, viscous and thermal characteristic lengths; its dynamic density
    and bulk modulus are fitted by ``num_poles`` Debye poles (half density,
    half modulus) at log-spaced relaxation times."""

    name: str = "porous"
    flow_resistivity: float = 10000.0
    porosity: float = 0.95
    tortuosity: float = 1.05
    viscous_length: float = 200e-6
    thermal_length: float = 400e-6
    thickness: float | None = None
    num_poles: int = 6
    rho_fluid: float = AIR_DENSITY
    eta: float = AIR_VISCOSITY
    Pr: float = AIR_PRANDTL
    gamma: float = AIR_GAMMA
    P0: float = AIR_PRESSURE
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        if self.flow_resistivity <= 0:
            raise ValueError("flow_resistivity must be positive")
        if not 0 < self.porosity <= 1:
            raise ValueError("porosity must be in (0, 1]")
        if self.tortuosity < 1:
            raise ValueError("tortuosity must be >= 1")
        if self.viscous_length <= 0:
            raise ValueError("viscous_length must be positive")
        if self.thermal_length <= 0:
            raise ValueError("thermal_length must be positive")
        if self.num_poles < 2:
            raise ValueError("num_poles must be >= 2")

    @property
    def rho_inf(self) -> float:  # rho_f alpha / phi
        return self.rho_fluid * self.tortuosity / self.porosity

    @property
    def K_inf(self) -> float:  # gamma P0 / phi
        return self.gamma * self.P0 / self.porosity

    @property
    def omega_viscous(self) -> float:
        return self.flow_resistivity * self.porosity / (self.rho_fluid * self.tortuosity)

    @property
    def omega_thermal(self) -> float:
        return self.eta / (self.rho_fluid * self.Pr * self.thermal_length**2)

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            self._poles_cache = self._fit_poles()
        return self._poles_cache

    def _fit_poles(self) -> list:
        """Relaxation times log-spaced over [1/(100 w_max), 1/(0.01 w_min)]
        of the viscous and thermal frequencies; strengths below 1e-6 are
        dropped (porous.py:155-204)."""
        w_lo = 0.01 * min(self.omega_viscous, self.omega_thermal)
        w_hi = 100 * max(self.omega_viscous, self.omega_thermal)
        n_rho = self.num_poles // 2
        out = []
        for target, n, response in (("density", n_rho, self._jca_density_normalized),
                                    ("modulus", self.num_poles - n_rho,
                                     self._jca_modulus_normalized)):
            tau = np.logspace(np.log10(1 / w_hi), np.log10(1 / w_lo), n)
            omega = np.logspace(1, 6, 100)
            chi = _debye_fit(tau, omega, response(omega))
            out += [Pole(pole_type=PoleType.DEBYE, delta_chi=d, tau=t, target=target)
                    for t, d in zip(tau, chi) if abs(d) > 1e-6]
        return out

    def _jca_density_normalized(self, omega):
        """rho / rho_inf of the Johnson model."""
        omega = np.asarray(omega) + 1e-20
        s, phi, a, L = self.flow_resistivity, self.porosity, self.tortuosity, self.viscous_length
        w_t = 4 * a**2 * self.eta * self.rho_fluid / (s**2 * L**2 * phi**2)
        return 1 + s * phi / (1j * omega * self.rho_fluid * a) * np.sqrt(1 + 1j * omega * w_t)

    def _jca_modulus_normalized(self, omega):
        """K / K_inf of the Champoux-Allard model."""
        omega = np.asarray(omega) + 1e-20
        L2 = self.thermal_length**2
        w_t = self.Pr * self.rho_fluid * L2 / (16 * self.eta)
        g = 1 + 8 * self.eta / (1j * omega * self.Pr * self.rho_fluid * L2) * np.sqrt(
            1 + 1j * omega * w_t)
        return self.gamma / (self.gamma - (self.gamma - 1) / g)

    def jca_density(self, omega):
        return self.rho_inf * self._jca_density_normalized(np.asarray(omega))

    def jca_modulus(self, omega):
        return self.K_inf * self._jca_modulus_normalized(np.asarray(omega))

    def jca_impedance(self, omega):
        return np.sqrt(self.jca_density(omega) * self.jca_modulus(omega))

    def jca_wavenumber(self, omega):
        omega = np.asarray(omega)
        return omega * np.sqrt(self.jca_density(omega) / self.jca_modulus(omega))

    def surface_impedance(self, omega, backing="rigid"):
        """Surface impedance of a layer of ``thickness`` on a rigid backing
        or on a backing impedance."""
        if self.thickness is None:
            raise ValueError("thickness must be set to compute surface impedance")
        omega = np.asarray(omega)
        zc, kd = self.jca_impedance(omega), self.jca_wavenumber(omega) * self.thickness
        if backing == "rigid":
            return -1j * zc / np.tan(kd)
        zb = float(backing)
        return zc * (zb + 1j * zc * np.tan(kd)) / (zc + 1j * zb * np.tan(kd))

    def absorption_coefficient_layer(self, omega, Z_air: float = 413.0, backing="rigid"):
        zs = self.surface_impedance(omega, backing)
        return 1 - np.abs((zs - Z_air) / (zs + Z_air)) ** 2

    def validate_pole_fit(self, omega, plot: bool = False) -> dict:
        """Relative error of the pole model against the exact JCA density and
        modulus at ``omega``."""
        if plot:
            raise NotImplementedError("plotting is not provided")
        e_rho = np.abs(self.effective_density(omega) - self.jca_density(omega)) / np.abs(
            self.jca_density(omega))
        e_k = np.abs(self.effective_modulus(omega) - self.jca_modulus(omega)) / np.abs(
            self.jca_modulus(omega))
        return {"density_max_error": float(np.max(e_rho)),
                "density_mean_error": float(np.mean(e_rho)),
                "modulus_max_error": float(np.max(e_k)),
                "modulus_mean_error": float(np.mean(e_k))}


@dataclass
class ViscoelasticSolid(AcousticMaterial):
    """Enclosure panel material as an effective fluid with Zener-type
    relaxation (solids.py:29-236): density, Young's modulus, loss factor at
    ``ref_frequency``; ``num_poles`` equal Debye modulus poles spread a
    decade either side of 1 / (2 pi f_ref) with total strength 2 eta."""

    name: str = "solid"
    density: float = 700.0
    youngs_modulus: float = 3.5e9
    loss_factor: float = 0.03
    poissons_ratio: float = 0.3
    ref_frequency: float = 1000.0
    num_poles: int = 3
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        if self.density <= 0:
            raise ValueError("density must be positive")
        if self.youngs_modulus <= 0:
            raise ValueError("youngs_modulus must be positive")
        if self.loss_factor < 0:
            raise ValueError("loss_factor must be non-negative")
        if not -1 < self.poissons_ratio < 0.5:
            raise ValueError("poissons_ratio must be in (-1, 0.5)")
        if self.ref_frequency <= 0:
            raise ValueError("ref_frequency must be positive")

    @property
    def bulk_modulus(self) -> float:
        return self.youngs_modulus / (3 * (1 - 2 * self.poissons_ratio))

    @property
    def shear_modulus(self) -> float:
        return self.youngs_modulus / (2 * (1 + self.poissons_ratio))

    @property
    def rho_inf(self) -> float:
        return self.density

    @property
    def K_inf(self) -> float:
        return self.bulk_modulus

    @property
    def longitudinal_modulus(self) -> float:
        return self.bulk_modulus + 4 * self.shear_modulus / 3

    @property
    def c_longitudinal(self) -> float:
        return np.sqrt(self.longitudinal_modulus / self.density)

    @property
    def relaxation_time(self) -> float:
        return 1 / (2 * np.pi * self.ref_frequency)

    @property
    def relaxation_strength(self) -> float:
        return 2 * self.loss_factor

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            tau0, total = self.relaxation_time, self.relaxation_strength
            if self.num_poles == 1:
                self._poles_cache = [Pole(pole_type=PoleType.DEBYE, delta_chi=total, tau=tau0,
                                          target="modulus")]
            else:
                taus = tau0 * np.logspace(-1, 1, self.num_poles)
                weights = np.ones(len(taus)) / len(taus)
                self._poles_cache = [Pole(pole_type=PoleType.DEBYE, delta_chi=total * w, tau=t,
                                          target="modulus")
                                     for t, w in zip(taus, weights) if w > 1e-6]
        return self._poles_cache

    def loss_factor_spectrum(self, omega):
        k = self.effective_modulus(omega)
        return np.imag(k) / np.real(k)

    def quality_factor(self, omega):
        return 1 / (self.loss_factor_spectrum(omega) + 1e-20)


@dataclass
class DampingMaterial(ViscoelasticSolid):
    """High-loss damping layer (butyl, sorbothane ...): five poles by
    default and a relaxation strength of min(3 eta, 0.9) (solids.py:239-278)."""

    poissons_ratio: float = 0.49
    num_poles: int = 5

    @property
    def relaxation_strength(self) -> float:
        return min(3 * self.loss_factor, 0.9)


@dataclass
class ImpedanceTube:
    """Normal-incidence absorption of a material in a two-microphone
    impedance tube (solids.py:281-385)."""

    length: float = 0.5
    diameter: float = 0.1
    mic_spacing: float = 0.05
    sample_distance: float = 0.1
    rho_air: float = 1.2
    c_air: float = 343.0

    @property
    def Z_air(self) -> float:
        return self.rho_air * self.c_air

    @property
    def max_frequency(self) -> float:  # first cross mode
        return 0.586 * self.c_air / self.diameter

    @property
    def min_frequency(self) -> float:
        return self.c_air / (20 * self.mic_spacing)

    def transfer_function_method(self, material, omega):
        """Complex reflection coefficient of the material's surface (a
        rigid-backed layer for a porous material with a thickness)."""
        omega = np.asarray(omega)
        if isinstance(material, PorousMaterial) and material.thickness is not None:
            zs = material.surface_impedance(omega, backing="rigid")
        else:
            zs = material.impedance(omega)
        return (zs - self.Z_air) / (zs + self.Z_air)

    def absorption_coefficient(self, material, omega):
        return 1 - np.abs(self.transfer_function_method(material, omega)) ** 2


class _AirAbsorber(AcousticMaterial):
    """Resonant absorbers in air: rho_inf and K_inf of the air, Lorentz
    modulus poles."""

    @property
    def rho_inf(self) -> float:
        return self.rho_air

    @property
    def K_inf(self) -> float:
        return self.rho_air * self.c_air**2

    def _lorentz(self, chi, w0, gamma):
        return Pole(pole_type=PoleType.LORENTZ, delta_chi=chi, omega_0=w0, gamma=gamma,
                    target="modulus")


@dataclass
class HelmholtzResonator(_AirAbsorber):
    """Helmholtz resonator as a material: one Lorentz modulus pole of
    strength -0.5 at f0 = c / (2 pi) sqrt(S / (V L_eff)), damping 2 eta w0
    (resonators.py:34-214)."""

    name: str = "helmholtz"
    neck_radius: float = 0.025
    neck_length: float = 0.05
    cavity_volume: float = 0.01
    loss_factor: float = 0.1
    end_correction: float = 0.85
    rho_air: float = AIR_DENSITY
    c_air: float = AIR_SPEED
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        for n in ("neck_radius", "neck_length", "cavity_volume"):
            if getattr(self, n) <= 0:
                raise ValueError(f"{n} must be positive")
        if self.loss_factor < 0:
            raise ValueError("loss_factor must be non-negative")

    @property
    def neck_area(self) -> float:
        return pi * self.neck_radius**2

    @property
    def effective_neck_length(self) -> float:
        return self.neck_length + 2 * self.end_correction * self.neck_radius

    @property
    def resonance_frequency(self) -> float:
        return self.c_air / (2 * pi) * np.sqrt(
            self.neck_area / (self.cavity_volume * self.effective_neck_length))

    @property
    def omega_0(self) -> float:
        return 2 * pi * self.resonance_frequency

    @property
    def acoustic_mass(self) -> float:
        return self.rho_air * self.effective_neck_length / self.neck_area

    @property
    def acoustic_compliance(self) -> float:
        return self.cavity_volume / (self.rho_air * self.c_air**2)

    @property
    def quality_factor_theoretical(self) -> float:
        return 2 * self.cavity_volume / (self.neck_area * (self.c_air / self.resonance_frequency))

    @property
    def gamma(self) -> float:
        return 2 * self.loss_factor * self.omega_0

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            self._poles_cache = [self._lorentz(-0.5, self.omega_0, self.gamma)]
        return self._poles_cache

    def impedance_analytical(self, omega):
        """R + i (w M - 1 / (w C)), R = eta w0 M."""
        omega = np.asarray(omega) + 1e-20
        m, c = self.acoustic_mass, self.acoustic_compliance
        return self.loss_factor * self.omega_0 * m + 1j * (omega * m - 1 / (omega * c))

    def absorption_analytical(self, omega):
        z, z0 = self.impedance_analytical(omega), self.rho_air * self.c_air
        return 1 - np.abs((z - z0) / (z + z0)) ** 2


@dataclass
class MembraneAbsorber(_AirAbsorber):
    """Panel absorber on an air cavity: one Lorentz pole of strength -0.3 at
    f0 = sqrt(rho c^2 / (m d)) / (2 pi) (resonators.py:217-317)."""

    name: str = "membrane"
    surface_density: float = 4.0
    cavity_depth: float = 0.1
    loss_factor: float = 0.15
    panel_area: float = 1.0
    rho_air: float = AIR_DENSITY
    c_air: float = AIR_SPEED
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        if self.surface_density <= 0:
            raise ValueError("surface_density must be positive")
        if self.cavity_depth <= 0:
            raise ValueError("cavity_depth must be positive")
        if self.loss_factor < 0:
            raise ValueError("loss_factor must be non-negative")

    @property
    def resonance_frequency(self) -> float:
        return (1 / (2 * pi)) * np.sqrt(
            self.rho_air * self.c_air**2 / (self.surface_density * self.cavity_depth))

    @property
    def omega_0(self) -> float:
        return 2 * pi * self.resonance_frequency

    @property
    def gamma(self) -> float:
        return 2 * self.loss_factor * self.omega_0

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            self._poles_cache = [self._lorentz(-0.3, self.omega_0, self.gamma)]
        return self._poles_cache


@dataclass
class PerforatedPanel(_AirAbsorber):
    """Perforated plate on a cavity: one Lorentz pole of strength
    -0.4 sqrt(eps) at f0 = c / (2 pi) sqrt(eps / (t_eff d))
    (resonators.py:320-477)."""

    name: str = "perforated"
    hole_diameter: float = 0.005
    plate_thickness: float = 0.01
    perforation_ratio: float = 0.1
    cavity_depth: float = 0.1
    loss_factor: float = 0.1
    rho_air: float = AIR_DENSITY
    c_air: float = AIR_SPEED
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        if self.hole_diameter <= 0:
            raise ValueError("hole_diameter must be positive")
        if self.plate_thickness <= 0:
            raise ValueError("plate_thickness must be positive")
        if not 0 < self.perforation_ratio < 1:
            raise ValueError("perforation_ratio must be in (0, 1)")
        if self.cavity_depth <= 0:
            raise ValueError("cavity_depth must be positive")

    @property
    def hole_radius(self) -> float:
        return self.hole_diameter / 2

    @property
    def effective_hole_length(self) -> float:
        corr = 0.85 * self.hole_radius * (1 - 1.47 * np.sqrt(self.perforation_ratio))
        return self.plate_thickness + 2 * max(corr, 0)

    @property
    def resonance_frequency(self) -> float:
        return self.c_air / (2 * pi) * np.sqrt(
            self.perforation_ratio / (self.effective_hole_length * self.cavity_depth))

    @property
    def omega_0(self) -> float:
        return 2 * pi * self.resonance_frequency

    @property
    def gamma(self) -> float:
        return 2 * self.loss_factor * self.omega_0

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            self._poles_cache = [self._lorentz(-0.4 * np.sqrt(self.perforation_ratio),
                                               self.omega_0, self.gamma)]
        return self._poles_cache

    def impedance_analytical(self, omega):
        """Viscous resistance of the holes, their mass and the cavity's
        stiffness, per unit open area."""
        omega = np.asarray(omega) + 1e-20
        eps, t_eff, d = self.perforation_ratio, self.effective_hole_length, self.cavity_depth
        k = omega / self.c_air
        mass = self.rho_air * t_eff / eps
        r = 32 * 1.81e-5 * self.plate_thickness / (eps * self.hole_radius**2)
        r *= 1 + self.loss_factor
        cavity = -1j * self.rho_air * self.c_air / np.tan(k * d) / eps
        return r + 1j * omega * mass + cavity


@dataclass
class QuarterWaveResonator(_AirAbsorber):
    """Closed tube: one Lorentz pole per mode n = 1 .. n_modes at
    (2n - 1) c / (4 L), strength -0.3 / n (resonators.py:480-580)."""

    name: str = "quarter_wave"
    length: float = 0.5
    diameter: float = 0.1
    loss_factor: float = 0.05
    n_modes: int = 3
    rho_air: float = AIR_DENSITY
    c_air: float = AIR_SPEED
    _poles_cache: list | None = field(default=None, repr=False)

    def __post_init__(self):
        if self.length <= 0:
            raise ValueError("length must be positive")
        if self.diameter <= 0:
            raise ValueError("diameter must be positive")
        if self.n_modes < 1:
            raise ValueError("n_modes must be >= 1")

    @property
    def area(self) -> float:
        return pi * (self.diameter / 2) ** 2

    def mode_frequency(self, n: int) -> float:
        return (2 * n - 1) * self.c_air / (4 * self.length)

    @property
    def fundamental_frequency(self) -> float:
        return self.mode_frequency(1)

    @property
    def poles(self) -> list:
        if self._poles_cache is None:
            out = []
            for n in range(1, self.n_modes + 1):
                w = 2 * pi * self.mode_frequency(n)
                out.append(self._lorentz(-0.3 / n, w, 2 * self.loss_factor * w))
            self._poles_cache = out
        return self._poles_cache
