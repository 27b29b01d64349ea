"""Reader of Lumol's TOML interactions input (lumol-input/src/interactions).

`InteractionsInput` mirrors the reference's reader: the same sections
(`[global]`, `[pairs]`, `[bonds]`, `[angles]`, `[dihedrals]`, `[charges]`,
`[coulomb]`), the same keys and units, the same defaults and the same error
messages, so that an interactions file written for Lumol sets up a `System`
of this engine the same way.  Sections are read in the reference's order
(mod.rs:53-62; charges before coulomb), and the entries of a section in
sorted key order, as the reference's TOML tables iterate.
"""
from __future__ import annotations

import tomllib

from . import system as _s
from .units import from_str as _unit


class InputError(Exception):
    """lumol_input::Error.  `kind` is "config" for a configuration error
    (Error::Config, whose text is the message) and "toml" for a TOML syntax
    error (Error::TOML)."""

    def __init__(self, message: str, kind: str = "config"):
        super().__init__(message)
        self.kind = kind

    @property
    def reason(self) -> str:
        return str(self)


def _is_int(v) -> bool:
    return isinstance(v, int) and not isinstance(v, bool)


def _is_number(v) -> bool:
    return _is_int(v) or isinstance(v, float)


def _debug_list(items) -> str:
    """Rust's `{:?}` of a Vec<&str>."""
    return "[" + ", ".join('"' + a.replace("\\", "\\\\").replace('"', '\\"') + '"' for a in items) + "]"


# ---- extract.rs -------------------------------------------------------------
def _str(key: str, table: dict, context: str) -> str:
    if key not in table:
        raise InputError(f"missing '{key}' key in {context}")
    v = table[key]
    if not isinstance(v, str):
        raise InputError(f"'{key}' must be a string in {context}")
    return v


def _number(key: str, table: dict, context: str) -> float:
    if key not in table:
        raise InputError(f"missing '{key}' key in {context}")
    v = table[key]
    if not _is_number(v):
        raise InputError(f"'{key}' must be a number in {context}")
    return float(v)


def _uint(key: str, table: dict, context: str) -> int:
    if key not in table:
        raise InputError(f"missing '{key}' key in {context}")
    v = table[key]
    if not _is_int(v) or v < 0:
        raise InputError(f"'{key}' must be a positive integer in {context}")
    return int(v)


def _typ(table: dict, context: str) -> str:
    if "type" not in table:
        raise InputError(f"missing 'type' key in {context}")
    v = table["type"]
    if not isinstance(v, str):
        raise InputError(f"'type' key must be a string in {context}")
    return v


def _value(text: str) -> float:
    try:
        return _unit(text)
    except ValueError as err:
        raise InputError(str(err)) from None


def _validate(config: dict) -> None:
    """lib.rs:76-95."""
    if "input" not in config:
        raise InputError("missing 'input' table")
    inp = config["input"]
    if not isinstance(inp, dict) or "version" not in inp:
        raise InputError("missing 'version' key in 'input' table")
    version = inp["version"]
    if not _is_int(version):
        raise InputError("'input.version' must be an integer")
    if version != 1:
        raise InputError(f"can only read version 1 of input, got version {version}")


def _restriction(table: dict):
    """read_restriction (interactions/mod.rs:65-102); None when absent."""
    if "restriction" not in table:
        return None
    r = table["restriction"]
    R = _s.PairRestriction
    if isinstance(r, str):
        names = {"none": R.NONE, "intramolecular": R.INTRA_MOLECULAR, "IntraMolecular": R.INTRA_MOLECULAR,
                 "intra-molecular": R.INTRA_MOLECULAR, "intermolecular": R.INTER_MOLECULAR,
                 "InterMolecular": R.INTER_MOLECULAR, "inter-molecular": R.INTER_MOLECULAR,
                 "exclude12": R.EXCLUDE12, "exclude13": R.EXCLUDE13, "exclude14": R.EXCLUDE14}
        if r in names:
            return names[r]
        if r == "scale14":
            raise InputError("'scale14' restriction must be a table")
        raise InputError(f"Unknown restriction '{r}'")
    if isinstance(r, dict):
        if len(r) != 1 or "scale14" not in r:
            raise InputError("Restriction table must be 'scale14'")
        if not isinstance(r["scale14"], float):
            raise InputError("'scale14' parameter must be a float")
        return R.scale14(r["scale14"])
    raise InputError("Restriction must be a table or a string")


# ---- potentials.rs ----------------------------------------------------------
def _harmonic(t):
    k = _str("k", t, "harmonic potential")
    x0 = _str("x0", t, "harmonic potential")
    return _s.Harmonic(k=_value(k), x0=_value(x0))


def _lennard_jones(t):
    sigma = _str("sigma", t, "Lennard-Jones potential")
    epsilon = _str("epsilon", t, "Lennard-Jones potential")
    return _s.LennardJones(sigma=_value(sigma), epsilon=_value(epsilon))


def _mie(t):
    sigma = _str("sigma", t, "Mie potential")
    epsilon = _str("epsilon", t, "Mie potential")
    m = _number("m", t, "Mie potential")
    n = _number("n", t, "Mie potential")
    return _s.Mie(_value(sigma), _value(epsilon), n, m)


def _cosine_harmonic(t):
    k = _str("k", t, "cosine harmonic potential")
    x0 = _str("x0", t, "cosine harmonic potential")
    return _s.CosineHarmonic(k=_value(k), x0=_value(x0))


def _torsion(t):
    n = _uint("n", t, "torsion potential")
    k = _str("k", t, "torsion potential")
    delta = _str("delta", t, "torsion potential")
    return _s.Torsion(k=_value(k), delta=_value(delta), n=n)


def _buckingham(t):
    a = _str("A", t, "Buckingham potential")
    c = _str("C", t, "Buckingham potential")
    rho = _str("rho", t, "Buckingham potential")
    return _s.Buckingham(_value(a), _value(c), _value(rho))


def _born(t):
    ctx = "Born-Mayer-Huggins potential"
    a, c, d = _str("A", t, ctx), _str("C", t, ctx), _str("D", t, ctx)
    rho, sigma = _str("rho", t, ctx), _str("sigma", t, ctx)
    return _s.BornMayerHuggins(_value(a), _value(c), _value(d), _value(sigma), _value(rho))


def _morse(t):
    a = _str("A", t, "Morse potential")
    depth = _str("depth", t, "Morse potential")
    x0 = _str("x0", t, "Morse potential")
    return _s.Morse(a=_value(a), x0=_value(x0), depth=_value(depth))


def _gaussian(t):
    a = _value(_str("A", t, "Gaussian potential"))
    b = _value(_str("B", t, "Gaussian potential"))
    if b <= 0.0:
        raise InputError("'B' parameter has to be positive in Gaussian potential")
    return _s.Gaussian(a, b)


def _null(_t):
    return _s.NullPotential()


_PAIR = {"null": _null, "harmonic": _harmonic, "lj": _lennard_jones, "buckingham": _buckingham, "born": _born,
         "morse": _morse, "gaussian": _gaussian, "mie": _mie}
_BOND = {"null": _null, "harmonic": _harmonic, "morse": _morse}
_ANGLE = {"null": _null, "harmonic": _harmonic, "cosine-harmonic": _cosine_harmonic, "morse": _morse}
_DIHEDRAL = {"null": _null, "harmonic": _harmonic, "cosine-harmonic": _cosine_harmonic, "torsion": _torsion,
             "morse": _morse}


def _potential(table: dict, readers: dict, context: str):
    typ = _typ(table, context)
    if typ not in readers:
        raise InputError(f"unknown potential type '{typ}'")
    return readers[typ](table)


def _computation(computation: dict, potential):
    """read_pair_computation (pairs.rs:191-202) and TableComputation's reader
    (potentials.rs:141-153)."""
    if len(computation) != 1:
        raise InputError("Missing computation type in computation table")
    (name,) = computation.keys()
    if name != "table":
        raise InputError(f"Unknown computation type '{name}'")
    table = computation["table"]
    if not isinstance(table, dict):
        raise InputError("'table' key in computation must be a TOML table")
    n = _uint("n", table, "table computation")
    max_ = _str("max", table, "table computation")
    return _s.TableComputation(potential, n, _value(max_))


def _wolf(t):
    return _s.Wolf(_value(_str("cutoff", t, "Wolf coulombic potential")))


def _ewald(t, system):
    """Ewald's reader (potentials.rs:163-191)."""
    ctx = "Ewald coulombic potential"
    cutoff = _value(_str("cutoff", t, ctx))
    if "accuracy" in t:
        if "kmax" in t or "alpha" in t:
            raise InputError("can not have both accuracy and kmax/alpha in Ewald coulombic potential")
        accuracy = _number("accuracy", t, ctx)
        return _s.Ewald.with_accuracy(cutoff, accuracy, system)
    kmax = _uint("kmax", t, ctx)
    alpha = _value(_str("alpha", t, ctx)) if "alpha" in t else None
    return _s.Ewald(cutoff, kmax, alpha)


class InteractionsInput:
    """lumol_input::InteractionsInput (interactions/mod.rs:21-63)."""

    def __init__(self, config: dict):
        self.config = config

    @classmethod
    def new(cls, path) -> "InteractionsInput":
        """Reads the interactions from the TOML file at `path`."""
        with open(path, encoding="utf-8") as f:
            return cls.from_str(f.read())

    @classmethod
    def from_str(cls, text: str) -> "InteractionsInput":
        try:
            config = tomllib.loads(text)
        except tomllib.TOMLDecodeError as err:
            raise InputError(str(err), kind="toml") from None
        _validate(config)
        return cls(config)

    def read(self, system) -> None:
        """Reads the interactions into `system` (mod.rs:53-62)."""
        self._read_pairs(system)
        self._read_bonds(system)
        self._read_angles(system)
        self._read_dihedrals(system)
        self._read_charges(system)
        self._read_coulomb(system)

    # ---- pairs.rs -----------------------------------------------------------
    def _global(self):
        """GlobalInformation::read (pairs.rs:22-53): (cutoff value, tail)."""
        if "global" not in self.config:
            return None, None
        g = self.config["global"]
        if not isinstance(g, dict):
            raise InputError("'global' section must be a table")
        tail = g.get("tail_correction")
        if tail is not None and not isinstance(tail, bool):
            raise InputError("the 'tail_correction' section must be a boolean value")
        return g.get("cutoff"), tail

    def _read_pairs(self, system) -> None:
        if "pairs" not in self.config:
            return
        pairs = self.config["pairs"]
        if not isinstance(pairs, dict):
            raise InputError("the 'pairs' section must be a table")
        global_cutoff, global_tail = self._global()
        for key in sorted(pairs):
            atoms = key.split("-")
            if len(atoms) != 2:
                raise InputError(f"expected two atoms for pair potential, got {len(atoms)} ({_debug_list(atoms)})")
            table = pairs[key]
            if not isinstance(table, dict):
                raise InputError(f"pair potential associated with {key} must be a table")
            potential = _potential(table, _PAIR, "pair potential")
            if "computation" in table:
                if not isinstance(table["computation"], dict):
                    raise InputError("'computation' section must be a table")
                potential = _computation(table["computation"], potential)
            cutoff = table["cutoff"] if "cutoff" in table else global_cutoff
            if cutoff is None:
                raise InputError("missing 'cutoff' value for pair potential")
            if isinstance(cutoff, str):
                interaction = _s.PairInteraction(potential, _value(cutoff))
            elif isinstance(cutoff, dict):
                if "shifted" not in cutoff:
                    raise InputError("'cutoff' table can only contain 'shifted' key")
                if not isinstance(cutoff["shifted"], str):
                    raise InputError("'cutoff.shifted' value must be a string")
                interaction = _s.PairInteraction.shifted(potential, _value(cutoff["shifted"]))
            else:
                raise InputError("'cutoff' must be a string or a table")
            tail = global_tail
            if "tail_correction" in table:
                tail = table["tail_correction"]
                if not isinstance(tail, bool):
                    raise InputError("the 'tail_correction' section must be a boolean value")
            if tail:
                interaction.enable_tail_corrections()
            restriction = _restriction(table)
            if restriction is not None:
                interaction.set_restriction(restriction)
            system.set_pair_potential((atoms[0], atoms[1]), interaction)

    def _read_bonds(self, system) -> None:
        if "bonds" not in self.config:
            return
        bonds = self.config["bonds"]
        if not isinstance(bonds, dict):
            raise InputError("the 'pairs' section must be a table")  # sic, pairs.rs:148-150
        for key in sorted(bonds):
            atoms = key.split("-")
            if len(atoms) != 2:
                raise InputError(f"expected two atoms for bond potential, got {len(atoms)} ({_debug_list(atoms)})")
            table = bonds[key]
            if not isinstance(table, dict):
                raise InputError(f"bond potential associated with {key} must be a table")
            system.set_bond_potential((atoms[0], atoms[1]), _potential(table, _BOND, "bond potential"))

    # ---- angles.rs ----------------------------------------------------------
    def _read_angles(self, system) -> None:
        if "angles" not in self.config:
            return
        angles = self.config["angles"]
        if not isinstance(angles, dict):
            raise InputError("the 'angles' section must be a table")
        for key in sorted(angles):
            atoms = key.split("-")
            if len(atoms) != 3:
                raise InputError(
                    f"expected three atoms for angle potential, got {len(atoms)} ({_debug_list(atoms)})")
            table = angles[key]
            if not isinstance(table, dict):
                raise InputError(f"angle potential associated with {key} must be a table")
            system.set_angle_potential(tuple(atoms), _potential(table, _ANGLE, "angle potential"))

    def _read_dihedrals(self, system) -> None:
        if "dihedrals" not in self.config:
            return
        dihedrals = self.config["dihedrals"]
        if not isinstance(dihedrals, dict):
            raise InputError("the 'dihedrals' section must be a table")
        for key in sorted(dihedrals):
            atoms = key.split("-")
            if len(atoms) != 4:
                raise InputError(
                    f"expected four atoms for dihedral potential, got {len(atoms)} ({_debug_list(atoms)})")
            table = dihedrals[key]
            if not isinstance(table, dict):
                raise InputError(f"dihedral potential associated with {key} must be a table")
            system.set_dihedral_potential(tuple(atoms), _potential(table, _DIHEDRAL, "dihedral potential"))

    # ---- coulomb.rs ---------------------------------------------------------
    def _read_coulomb(self, system) -> None:
        if "coulomb" not in self.config:
            return
        coulomb = self.config["coulomb"]
        if not isinstance(coulomb, dict):
            raise InputError("the 'coulomb' section must be a table")
        solvers = sorted(k for k in coulomb if k != "restriction")
        if len(solvers) != 1:
            raise InputError("got more than one coulombic solver: " + " and ".join(solvers))
        key = solvers[0]
        table = coulomb[key]
        if not isinstance(table, dict):
            raise InputError(f"coulombic solver '{key}' must be a table")
        if key == "wolf":
            potential = _wolf(table)
        elif key == "ewald":
            potential = _ewald(table, system)
        else:
            raise InputError(f"unknown coulomb solver '{key}'")
        restriction = _restriction(coulomb)
        if restriction is not None:
            potential.set_restriction(restriction)
        system.set_coulomb_potential(potential)

    def _read_charges(self, system) -> None:
        if "charges" not in self.config:
            return
        charges = self.config["charges"]
        if not isinstance(charges, dict):
            raise InputError("the 'charges' section must be a table")
        for name in sorted(charges):
            q = charges[name]
            if not _is_number(q):
                raise InputError("charges must be numbers")
            for i, particle in enumerate(system.names):
                if particle == name:
                    system.set_charge(i, float(q))


def read_interactions(system, path) -> None:
    """System::read_interactions-style helper: InteractionsInput::new(path).read(system)."""
    InteractionsInput.new(path).read(system)
