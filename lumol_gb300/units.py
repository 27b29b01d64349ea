"""Conversion to Lumol's internal units (lumol-core/src/units.rs).

Internal units: Angstrom, femtosecond, unified atomic mass, Kelvin, radian;
energy is 1e-4 kJ/mol.  `from_(value, "kJ/mol/A^2")` mirrors `units::from`.
Unit expressions are products and quotients of the units below with integer
powers, evaluated left to right.
"""
from __future__ import annotations

import math
import re

# lumol-core/src/consts.rs:9-15 and units.rs:29-74
K_BOLTZMANN = 8.31446284161522e-7
FOUR_PI_EPSILON_0 = 7.197589831304046
BOHR_RADIUS = 0.52917720859
AVOGADRO_NUMBER = 6.02214179e23
U_IN_KG = 1.660538782e-27

CONVERSION_FACTORS = {
    "A": 1.0, "nm": 10.0, "pm": 1e-2, "fm": 1e-5, "m": 1e10, "bohr": BOHR_RADIUS,
    "fs": 1.0, "ps": 1e3, "ns": 1e6,
    "u": 1.0, "Da": 1.0, "kDa": 1.0, "g": 1e-3 / U_IN_KG, "kg": 1.0 / U_IN_KG,
    "K": 1.0,
    "mol": AVOGADRO_NUMBER,
    "rad": 1.0, "deg": math.pi / 180.0,
    "J": 1e-10 / U_IN_KG, "kJ": 1e-7 / U_IN_KG, "kcal": 4.184 * 1e-7 / U_IN_KG,
    "eV": 1.60217653e-19 * 1e-10 / U_IN_KG, "H": 4.35974417e-18 * 1e-10 / U_IN_KG,
    "Ry": 4.35974417e-18 / 2.0 * 1e-10 / U_IN_KG,
    "N": 1e-20 / U_IN_KG,
    "Pa": 1e-40 / U_IN_KG, "kPa": 1e-37 / U_IN_KG, "MPa": 1e-34 / U_IN_KG,
    "bar": 1e-35 / U_IN_KG, "atm": 101325.0 * 1e-40 / U_IN_KG,
}

_TOKEN = re.compile(r"\s*([A-Za-z]+)(?:\^(-?\d+))?\s*([*/]|$)")


def _factor(unit: str) -> float:
    factor = 1.0
    op = "*"
    pos = 0
    unit = unit.strip()
    while pos < len(unit):
        m = _TOKEN.match(unit, pos)
        if not m or m.end() == pos:
            raise ValueError(f"can not parse unit '{unit}'")
        name, power, nxt = m.group(1), m.group(2), m.group(3)
        if name not in CONVERSION_FACTORS:
            raise ValueError(f"unknown unit '{name}'")
        value = CONVERSION_FACTORS[name] ** (int(power) if power else 1)
        factor = factor * value if op == "*" else factor / value
        op = nxt or "*"
        pos = m.end()
    return factor


def from_(value: float, unit: str) -> float:
    """Converts `value` in `unit` to internal units (units::from)."""
    return value * _factor(unit)


def to(value: float, unit: str) -> float:
    """Converts `value` in internal units to `unit` (units::to)."""
    return value / _factor(unit)


# Atomic masses of the elements the engine's workloads use
# (lumol-core/src/sys/config/mass.rs:8-25).
ATOMIC_MASSES = {
    "H": 1.008, "He": 4.002602, "C": 12.011, "N": 14.007, "O": 15.999, "F": 18.9984032,
    "Ne": 20.1797, "Na": 22.98976928, "Cl": 35.45, "Ar": 39.948, "Kr": 83.798, "Xe": 131.293,
}
