"""Unit system and physical constants of mdpy, restated in FP64.

mdpy works in Angstrom / Dalton / femtosecond / elementary charge / Kelvin
(mdpy/unit/__init__.py:31-49); the derived energy unit is Da*A^2/fs^2
(= 1e4 kJ/mol).  Every constant below is computed from the same SI inputs
the reference uses, so values agree with mdpy's to float32 rounding (mdpy
stores ``Quantity`` values as float32, mdpy/unit/quantity.py:32-36):

* KB       = 1.38064852e-23 J/K              (mdpy/unit/__init__.py:54)
* NA       = 6.0221e23 /mol                  (mdpy/unit/__init__.py:55; not CODATA)
* EPSILON0 = 8.85418e-12 s^2 C^2 m^-3 kg^-1  (mdpy/unit/__init__.py:56-58)
* Dalton   = 1.66053904e-27 kg               (mdpy/unit/unit_definition.py:54)
* e        = 1.602176634e-19 C               (mdpy/unit/unit_definition.py:90)
* kcal/mol = 4.184e3 / 6.0221e23 J           (mdpy/unit/unit_definition.py:117)

Only plain numbers (already in the default units) and objects exposing
mdpy's ``Quantity`` interface (``convert_to(unit).value``) are accepted by
:func:`check_quantity_value`; the dimensional algebra of mdpy.unit itself is
host-side set-up and is not rebuilt here.
"""
from __future__ import annotations

import math

import numpy as np

# --- SI inputs, exactly as mdpy states them --------------------------------
_KB_SI = 1.38064852e-23
_NA = 6.0221e23
_EPS0_SI = 8.85418e-12
_DALTON_KG = 1.66053904e-27
_E_C = 1.602176634e-19
_ANGSTROM_M = 1e-10
_FS_S = 1e-15

# --- derived internal units -------------------------------------------------
#: one internal energy unit (Da*A^2/fs^2) in joule
ENERGY_UNIT_J = _DALTON_KG * _ANGSTROM_M**2 / _FS_S**2
#: kcal/mol expressed in internal energy units
KCAL_PER_MOL = 4.184e3 / _NA / ENERGY_UNIT_J
#: kJ/mol expressed in internal energy units
KJ_PER_MOL = 1.0e3 / _NA / ENERGY_UNIT_J
#: Boltzmann constant in internal energy units per Kelvin
KB = _KB_SI / ENERGY_UNIT_J
#: vacuum permittivity in e^2 fs^2 / (Da A^3)
EPSILON0 = _EPS0_SI * _DALTON_KG / _E_C**2
#: Coulomb constant 1/(4 pi eps0) in internal energy * A / e^2
COULOMB_K = 1.0 / (4.0 * math.pi * EPSILON0)
#: nanoseconds per femtosecond
NS_PER_FS = 1e-6


def check_quantity_value(val, unit_name: str | None = None):
    """Return ``val`` as a plain float/ndarray in mdpy's default units.

    Mirrors ``mdpy.utils.check_quantity_value`` (mdpy/utils/check_quantity.py:21-27):
    ``None`` passes through, plain numbers are taken to be in the default
    unit, and an object with mdpy's ``Quantity`` interface is converted with
    its own ``convert_to`` when ``unit_name`` names an attribute of
    ``mdpy.unit`` (so a user of the reference can pass their quantities in).
    """
    if val is None:
        return None
    if hasattr(val, "convert_to") and hasattr(val, "value"):
        if unit_name is None:
            raise TypeError("a Quantity needs a target unit name")
        import importlib

        mdunit = importlib.import_module("mdpy.unit")
        return val.convert_to(getattr(mdunit, unit_name)).value
    if isinstance(val, np.ndarray):
        return val
    return float(val)


def kinetic_temperature(kinetic_energy: float, num_particles: int) -> float:
    """Temperature from kinetic energy, T = 2 KE / (3 N kB), as LogDumper
    reports it (mdpy/dumper/log_dumper.py:160-164)."""
    return 2.0 * kinetic_energy / (3.0 * num_particles * KB)


def ns_per_day(steps_per_second: float, time_step_fs: float) -> float:
    """Simulation speed as LogDumper defines it (mdpy/dumper/log_dumper.py:199-208)."""
    return steps_per_second * time_step_fs * NS_PER_FS * 86400.0
