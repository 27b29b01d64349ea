"""Conversion to Lumol's internal units (lumol-core/src/units.rs).

Internal units: Angstrom, femtosecond, unified atomic mass, Kelvin, radian;
energy is u A^2 / fs^2 = 1e4 kJ/mol (the module comment of units.rs says
1e-4 kJ/mol; its conversion factors give 1e4).  `from_(value, "kJ/mol/A^2")` mirrors `units::from`.
Unit expressions are products and quotients of the units below with integer
powers and parentheses.
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

_TOKEN = re.compile(r"\s*(?:([*/^()])|([^*/^()\s]+))")


def _tokens(unit: str) -> list[str]:
    out, pos = [], 0
    while pos < len(unit):
        m = _TOKEN.match(unit, pos)
        if m is None:  # only whitespace is left
            break
        out.append(m.group(1) or m.group(2))
        pos = m.end()
    return out


def _factor(unit: str) -> float:
    """Evaluates a unit expression as units.rs:183-365 reads it: names,
    '*' and '/' (left-associative, same precedence), '^' with an integer power
    (higher precedence), and parentheses."""
    toks = _tokens(unit)
    pos = 0

    def peek():
        return toks[pos] if pos < len(toks) else None

    def atom() -> float:
        nonlocal pos
        t = peek()
        if t is None:
            raise ValueError(f"malformed unit '{unit}': missing a value")
        pos += 1
        if t == "(":
            v = expr()
            if peek() != ")":
                raise ValueError(f"malformed unit '{unit}': unbalanced parenthesis")
            pos += 1
            return v
        if t in "*/^)":
            raise ValueError(f"malformed unit '{unit}': unexpected '{t}'")
        if t not in CONVERSION_FACTORS:
            raise ValueError(f"unknown unit '{t}'")
        return CONVERSION_FACTORS[t]

    def power() -> float:
        nonlocal pos
        v = atom()
        while peek() == "^":
            pos += 1
            t = peek()
            try:
                exponent = int(t)
            except (TypeError, ValueError):
                raise ValueError(f"malformed unit '{unit}': invalid value after ^: {t}") from None
            pos += 1
            v = v ** exponent
        return v

    def expr() -> float:
        nonlocal pos
        v = power()
        while peek() in ("*", "/"):
            op = toks[pos]
            pos += 1
            rhs = power()
            v = v * rhs if op == "*" else v / rhs
        return v

    value = expr()
    if pos != len(toks):
        raise ValueError(f"malformed unit '{unit}': remaining values after the end of the unit: "
                         + " ".join(toks[pos:]))
    return value


def from_str(value: str) -> float:
    """units::from_str (units.rs:384-394): "<number> <unit>" to internal
    units; the unit may be omitted."""
    parts = value.split()
    if not parts:
        raise ValueError("can not parse an empty value")
    factor = _factor(" ".join(parts[1:])) if len(parts) > 1 else 1.0
    try:
        number = float(parts[0])
    except ValueError:
        raise ValueError(f"can not parse '{parts[0]}' as a number") from None
    return factor * number


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
