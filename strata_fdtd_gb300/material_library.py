"""Predefined materials (materials/library.py of rjwalters/strata-fdtd): air
and water, porous absorbers, enclosure woods and damping layers, with the
reference's parameters, and the registry functions that look them up."""
from __future__ import annotations

from .material_models import DampingMaterial, PorousMaterial, ViscoelasticSolid
from .materials import AIR_20C, SimpleMaterial

AIR_25C = SimpleMaterial(name="air_25C", _rho=1.184, _c=346.3)
AIR_15C = SimpleMaterial(name="air_15C", _rho=1.225, _c=340.3)
WATER_20C = SimpleMaterial(name="water_20C", _rho=998.2, _c=1482.0)


def _porous(name, sigma, phi, alpha, lv, lt):
    return PorousMaterial(name=name, flow_resistivity=sigma, porosity=phi, tortuosity=alpha,
                          viscous_length=lv, thermal_length=lt, num_poles=6)


# name, flow resistivity (Pa s/m^2), porosity, tortuosity, viscous and thermal lengths (m)
FIBERGLASS_24 = _porous("fiberglass_24kg", 8000, 0.99, 1.02, 200e-6, 400e-6)
FIBERGLASS_32 = _porous("fiberglass_32kg", 14000, 0.98, 1.03, 150e-6, 300e-6)
FIBERGLASS_48 = _porous("fiberglass_48kg", 25000, 0.98, 1.04, 100e-6, 200e-6)
FIBERGLASS_96 = _porous("fiberglass_96kg", 60000, 0.96, 1.06, 60e-6, 120e-6)
MINERAL_WOOL_40 = _porous("mineral_wool_40kg", 20000, 0.97, 1.04, 80e-6, 160e-6)
MINERAL_WOOL_60 = _porous("mineral_wool_60kg", 35000, 0.96, 1.05, 60e-6, 120e-6)
MINERAL_WOOL_100 = _porous("mineral_wool_100kg", 70000, 0.94, 1.08, 40e-6, 80e-6)
ACOUSTIC_FOAM_OPEN = _porous("acoustic_foam_open", 12000, 0.97, 1.10, 150e-6, 300e-6)
ACOUSTIC_FOAM_DENSE = _porous("acoustic_foam_dense", 30000, 0.95, 1.15, 80e-6, 160e-6)
POLYURETHANE_FOAM = _porous("polyurethane_foam", 15000, 0.98, 1.08, 120e-6, 240e-6)
POLYESTER_BATTING = _porous("polyester_batting", 5000, 0.99, 1.01, 300e-6, 600e-6)
WOOL_FELT = _porous("wool_felt", 30000, 0.95, 1.30, 80e-6, 160e-6)
COTTON_BATTING = _porous("cotton_batting", 8000, 0.98, 1.05, 200e-6, 400e-6)


def _solid(name, rho, e, eta, nu):
    return ViscoelasticSolid(name=name, density=rho, youngs_modulus=e, loss_factor=eta,
                             poissons_ratio=nu, num_poles=3)


# name, density (kg/m^3), Young's modulus (Pa), loss factor, Poisson's ratio
MDF_LIGHT = _solid("MDF_light", 600, 2.8e9, 0.035, 0.25)
MDF_MEDIUM = _solid("MDF_medium", 720, 3.5e9, 0.030, 0.25)
MDF_HIGH = _solid("MDF_high", 850, 4.2e9, 0.025, 0.25)
PLYWOOD_BIRCH = _solid("plywood_birch", 680, 12.0e9, 0.015, 0.35)
PLYWOOD_MARINE = _solid("plywood_marine", 700, 10.0e9, 0.020, 0.30)
PLYWOOD_SOFTWOOD = _solid("plywood_softwood", 550, 8.0e9, 0.020, 0.35)
PARTICLE_BOARD = _solid("particle_board", 650, 2.5e9, 0.040, 0.25)
OSB = _solid("OSB", 620, 4.5e9, 0.025, 0.30)
HARDWOOD_OAK = _solid("hardwood_oak", 750, 12.5e9, 0.010, 0.35)


def _damping(name, rho, e, eta):
    return DampingMaterial(name=name, density=rho, youngs_modulus=e, loss_factor=eta,
                           poissons_ratio=0.49, num_poles=5)


BUTYL_RUBBER = _damping("butyl_rubber", 1200, 1.0e6, 0.40)
NEOPRENE = _damping("neoprene", 1300, 2.0e6, 0.15)
SORBOTHANE = _damping("sorbothane", 1100, 0.5e6, 0.50)
EPDM_RUBBER = _damping("EPDM_rubber", 1150, 3.0e6, 0.12)
SILICONE_RUBBER = _damping("silicone_rubber", 1100, 1.5e6, 0.08)


def _by_name(*mats):
    return {m.name: m for m in mats}


MATERIALS = {
    "fluids": _by_name(AIR_20C, AIR_25C, AIR_15C, WATER_20C),
    "fiberglass": _by_name(FIBERGLASS_24, FIBERGLASS_32, FIBERGLASS_48, FIBERGLASS_96),
    "mineral_wool": _by_name(MINERAL_WOOL_40, MINERAL_WOOL_60, MINERAL_WOOL_100),
    "foam": _by_name(ACOUSTIC_FOAM_OPEN, ACOUSTIC_FOAM_DENSE, POLYURETHANE_FOAM),
    "fibrous": _by_name(POLYESTER_BATTING, WOOL_FELT, COTTON_BATTING),
    "mdf": _by_name(MDF_LIGHT, MDF_MEDIUM, MDF_HIGH),
    "plywood": _by_name(PLYWOOD_BIRCH, PLYWOOD_MARINE, PLYWOOD_SOFTWOOD),
    "other_wood": _by_name(PARTICLE_BOARD, OSB, HARDWOOD_OAK),
    "damping": _by_name(BUTYL_RUBBER, NEOPRENE, SORBOTHANE, EPDM_RUBBER, SILICONE_RUBBER),
}


def get_material(name: str):
    """The library material of that name (case-insensitive)."""
    for category in MATERIALS.values():
        for key, mat in category.items():
            if key.lower() == name.lower():
                return mat
    raise KeyError(f"Material '{name}' not found. Use list_materials() to see available "
                   "materials.")


def list_materials(category: str | None = None) -> list[str]:
    if category is not None:
        if category not in MATERIALS:
            raise KeyError(f"Unknown category '{category}'. Available: {list(MATERIALS.keys())}")
        return list(MATERIALS[category])
    return [name for cat in MATERIALS.values() for name in cat]


def list_categories() -> list[str]:
    return list(MATERIALS)


def material_summary(name: str) -> str:
    return get_material(name).summary()
