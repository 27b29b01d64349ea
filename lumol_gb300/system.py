"""Host-side mirror of Lumol's System / potential / integrator interface.

The classes keep the names, arguments and error behaviour of lumol-core and
lumol-sim, so that a simulation written against Lumol maps onto them line by
line; every computation runs on the GPU through the C ABI of
include/lumol_gb300.h (see `_capi.py`).  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _capi as C
from .units import ATOMIC_MASSES, FOUR_PI_EPSILON_0


# ---------------------------------------------------------------------------
# Restrictions (lumol-core/src/energy/restrictions.rs:13-33)
# ---------------------------------------------------------------------------
class PairRestriction:
    NONE = 0
    INTRA_MOLECULAR = 1
    INTER_MOLECULAR = 2
    EXCLUDE12 = 3
    EXCLUDE13 = 4
    EXCLUDE14 = 5

    @staticmethod
    def scale14(factor: float) -> tuple:
        return (6, float(factor))


def _restriction(r) -> tuple[int, float]:
    if isinstance(r, tuple):
        return int(r[0]), float(r[1])
    return int(r), 1.0


# ---------------------------------------------------------------------------
# Potentials (lumol-core/src/energy/functions.rs)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class NullPotential:
    """NullPotential (functions.rs:29-50)."""

    def _params(self):
        return C.LG_PAIR_NULL, (0.0, 0.0, 0.0)


@dataclass(frozen=True)
class LennardJones:
    """LennardJones {sigma, epsilon} (functions.rs:71-107)."""
    sigma: float
    epsilon: float

    def _params(self):
        return C.LG_PAIR_LJ, (self.sigma, self.epsilon, 0.0)


@dataclass(frozen=True)
class Buckingham:
    """Buckingham {a, c, rho}: A exp(-r / rho) - C / r^6 (functions.rs:276-319)."""
    a: float
    c: float
    rho: float

    def _params(self):
        return C.LG_PAIR_BUCKINGHAM, (self.a, self.c, self.rho)


@dataclass(frozen=True)
class Harmonic:
    """Harmonic {k, x0}: k / 2 (x - x0)^2 (functions.rs:127-160)."""
    k: float
    x0: float

    def _params(self):
        return C.LG_PAIR_HARMONIC, (self.k, self.x0, 0.0)


@dataclass(frozen=True)
class CosineHarmonic:
    """CosineHarmonic::new(k, x0): k / 2 (cos x - cos x0)^2, for angles and
    dihedral angles (functions.rs:162-210)."""
    k: float
    x0: float

    def _params(self):
        return C.LG_BONDED_COSINE_HARMONIC, (self.k, self.x0, 0.0)


@dataclass(frozen=True)
class Torsion:
    """Torsion {k, delta, n}: k (1 + cos(n phi - delta)), for dihedral angles
    (functions.rs:212-258)."""
    k: float
    delta: float
    n: int

    def _params(self):
        return C.LG_BONDED_TORSION, (self.k, self.delta, self.n)


@dataclass(frozen=True)
class BornMayerHuggins:
    """BornMayerHuggins {a, c, d, sigma, rho}:
    A exp((sigma - r) / rho) - C / r^6 + D / r^8 (functions.rs:321-386)."""
    a: float
    c: float
    d: float
    sigma: float
    rho: float

    def _params(self):
        return C.LG_PAIR_BMH, (self.a, self.c, self.d, self.sigma, self.rho)


@dataclass(frozen=True)
class Morse:
    """Morse {a, x0, depth}: depth (1 - exp(a (x0 - r)))^2 (functions.rs:388-437)."""
    a: float
    x0: float
    depth: float

    def _params(self):
        return C.LG_PAIR_MORSE, (self.a, self.x0, self.depth)


@dataclass(frozen=True)
class Gaussian:
    """Gaussian::new(a, b): -a exp(-b r^2), b > 0 (functions.rs:439-494)."""
    a: float
    b: float

    def __post_init__(self):
        if not self.b > 0.0:
            raise ValueError('"b" has to be positive in Gaussian potential')

    def _params(self):
        return C.LG_PAIR_GAUSSIAN, (self.a, self.b)


@dataclass(frozen=True)
class Mie:
    """Mie::new(sigma, epsilon, n, m): the LJ form with exponents n > m
    (functions.rs:496-592)."""
    sigma: float
    epsilon: float
    n: float
    m: float

    def __post_init__(self):
        if not self.m < self.n:
            raise ValueError("The repulsive exponent n has to be larger than the attractive exponent m")

    def _params(self):
        return C.LG_PAIR_MIE, (self.sigma, self.epsilon, self.n, self.m)


class TableComputation:
    """TableComputation::new(potential, size, max) (energy/computations.rs:63-173):
    the potential's energy and force tabulated at r = i max / size,
    interpolated linearly, zero from the last point on; the tail corrections
    are the potential's own."""

    def __init__(self, potential, size: int, max: float):
        if size <= 0 or not max > 0.0:
            raise ValueError("TableComputation needs a positive size and maximum")
        self.potential = potential
        self._table = (int(size), float(max))

    def _params(self):
        return self.potential._params()


class PairInteraction:
    """PairInteraction (lumol-core/src/energy/pairs.rs:22-296)."""

    def __init__(self, potential, cutoff: float):
        self.potential = potential
        self.cutoff = float(cutoff)
        self.shifted_energy = False
        self.tail = False
        self.restriction = PairRestriction.NONE

    @classmethod
    def shifted(cls, potential, cutoff: float) -> "PairInteraction":
        p = cls(potential, cutoff)
        p.shifted_energy = True
        return p

    def enable_tail_corrections(self) -> None:
        self.tail = True

    def set_restriction(self, restriction) -> None:
        self.restriction = restriction

    def _lower(self) -> C.LgPair:
        kind, params = self.potential._params()
        p0, p1, p2, p3, p4 = (list(params) + [0.0] * 5)[:5]
        r, s14 = _restriction(self.restriction)
        tsize, tmax = getattr(self.potential, "_table", (0, 0.0))
        return C.LgPair(kind, int(self.shifted_energy), r, int(self.tail), p0, p1, p2, self.cutoff, s14, p3, p4,
                        tsize, 0, tmax)


class Ewald:
    """Ewald::new(cutoff, kmax, alpha) (energy/global/ewald.rs:278-305), used
    as SharedEwald behind System::set_coulomb_potential."""

    def __init__(self, cutoff: float, kmax: int, alpha: float | None = None):
        import math
        a = math.pi / cutoff if alpha is None else alpha
        if cutoff < 0.0:
            raise ValueError("the cutoff can not be negative in Ewald")
        if a < 0.0:
            raise ValueError("alpha can not be negative in Ewald")
        if kmax == 0:
            raise ValueError("kmax can not be 0 in Ewald")
        self.cutoff = float(cutoff)
        self.kmax = int(kmax)
        self.alpha = float(a)
        self.restriction = PairRestriction.NONE

    @classmethod
    def with_accuracy(cls, cutoff: float, accuracy: float, system: "System") -> "Ewald":
        """Ewald::with_accuracy (ewald.rs:312-351): alpha from the accuracy, the
        cutoff, the particle count, the cell volume and the charges; kmax the
        smallest one whose k-space error estimate is within the accuracy."""
        if cutoff < 0.0:
            raise ValueError("the cutoff can not be negative in Ewald")
        if accuracy < 0.0:
            raise ValueError("accuracy can not be negative in Ewald")
        f = np.float64
        with np.errstate(all="ignore"):  # IEEE arithmetic: an empty or neutral system gives inf / NaN
            q2 = f(0.0)
            for q in system.charges:
                q2 += f(q) * f(q)
            q2 /= f(FOUR_PI_EPSILON_0)
            natoms = f(system.size)
            a, b, c = (f(x) for x in system.cell.lengths)
            alpha = f(accuracy) * np.sqrt(natoms * f(cutoff) * a * b * c) / (f(2.0) * q2)
            if alpha >= 1.0:
                alpha = (f(1.35) - f(0.15) * np.log(f(accuracy))) / f(cutoff)
            else:
                alpha = np.sqrt(-np.log(alpha)) / f(cutoff)
            min_length = min(a, b, c)

            def error(kmax: float):
                arg = f(np.pi) * f(kmax) / (alpha * min_length)
                return f(1.1283791670955126) * q2 * alpha / min_length / np.sqrt(f(kmax) * natoms) * np.exp(-arg * arg)

            kmax = 1
            while error(kmax) > accuracy:  # 2 / sqrt(pi) above is f64's FRAC_2_SQRT_PI
                kmax += 1
        alpha = float(alpha)
        return cls(cutoff, kmax, alpha)

    def set_restriction(self, restriction) -> None:
        self.restriction = restriction

    def _lower(self) -> C.LgCoulomb:
        r, s14 = _restriction(self.restriction)
        return C.LgCoulomb(C.LG_COULOMB_EWALD, r, self.kmax, 0, self.cutoff, self.alpha, s14)


class Wolf:
    """Wolf::new(cutoff) (energy/global/wolf.rs:68-84)."""

    def __init__(self, cutoff: float):
        if not cutoff > 0.0:
            raise ValueError("Got a negative cutoff in Wolf summation")
        self.cutoff = float(cutoff)
        self.restriction = PairRestriction.NONE

    def set_restriction(self, restriction) -> None:
        self.restriction = restriction

    def _lower(self) -> C.LgCoulomb:
        r, s14 = _restriction(self.restriction)
        return C.LgCoulomb(C.LG_COULOMB_WOLF, r, 0, 0, self.cutoff, 0.0, s14)


def _cross(x, y):
    """Vector3D ^ (types/vectors.rs:219-228)."""
    return (x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0])


def _dot(x, y):
    """Vector3D * Vector3D (types/vectors.rs:212-217)."""
    return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]


def _mat_vec(m, v):
    """Matrix3 * Vector3D (types/matrix.rs:389-398), row by row."""
    return tuple(m[a][0] * v[0] + m[a][1] * v[1] + m[a][2] * v[2] for a in range(3))


def _mat_mul(x, y):
    """Matrix3 * Matrix3 (types/matrix.rs:342-362)."""
    return tuple(tuple(x[i][0] * y[0][j] + x[i][1] * y[1][j] + x[i][2] * y[2][j] for j in range(3))
                 for i in range(3))


def _inverse(m):
    """Matrix3::inverse (types/matrix.rs:212-249)."""
    det = (m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
           + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]))
    if not abs(det) > 1e-30:
        raise ValueError("The matrix is not invertible!")
    i = 1.0 / det
    return ((((m[1][1] * m[2][2] - m[2][1] * m[1][2]) * i), ((m[0][2] * m[2][1] - m[0][1] * m[2][2]) * i),
             ((m[0][1] * m[1][2] - m[0][2] * m[1][1]) * i)),
            (((m[1][2] * m[2][0] - m[1][0] * m[2][2]) * i), ((m[0][0] * m[2][2] - m[0][2] * m[2][0]) * i),
             ((m[1][0] * m[0][2] - m[0][0] * m[1][2]) * i)),
            (((m[1][0] * m[2][1] - m[2][0] * m[1][1]) * i), ((m[2][0] * m[0][1] - m[0][0] * m[2][1]) * i),
             ((m[0][0] * m[1][1] - m[1][0] * m[0][1]) * i)))


class UnitCell:
    """UnitCell (lumol-core/src/sys/config/cells.rs): an orthorhombic or a
    triclinic cell, held as its matrix (columns: the cell vectors) and shape.
    `lengths` are the distances between opposite faces (UnitCell::lengths,
    cells.rs:134-146: a, b, c for an orthorhombic cell), which the cutoff
    checks read."""

    ORTHORHOMBIC, TRICLINIC = "orthorhombic", "triclinic"

    def __init__(self, matrix, shape: str = "orthorhombic"):
        m = tuple(tuple(float(x) for x in row) for row in np.asarray(matrix, dtype=np.float64).reshape(3, 3))
        if shape not in (self.ORTHORHOMBIC, self.TRICLINIC):
            raise ValueError(f"unknown cell shape {shape!r}")
        self._m = m
        self.shape = shape
        self._inv = _inverse(m)
        va, vb, vc = ((m[0][k], m[1][k], m[2][k]) for k in range(3))

        def face(x, y, v):  # (x ^ y).normalized(), then |n * v|
            n = _cross(x, y)
            norm = float(np.sqrt(_dot(n, n)))
            n = (n[0] / norm, n[1] / norm, n[2] / norm)
            return abs(_dot(n, v))
        self.lengths = (face(vb, vc, va), face(vc, va, vb), face(va, vb, vc))

    @classmethod
    def cubic(cls, length: float) -> "UnitCell":
        if not length > 0.0:
            raise ValueError("Cell lengths must be positive")
        return cls(np.diag([float(length)] * 3))

    @classmethod
    def ortho(cls, a: float, b: float, c: float) -> "UnitCell":
        if not (a > 0.0 and b > 0.0 and c > 0.0):
            raise ValueError("Cell lengths must be positive")
        return cls(np.diag([float(a), float(b), float(c)]))

    @classmethod
    def triclinic(cls, a: float, b: float, c: float, alpha: float, beta: float, gamma: float) -> "UnitCell":
        """UnitCell::triclinic (cells.rs:72-94): angles in degrees."""
        if not (a > 0.0 and b > 0.0 and c > 0.0):
            raise ValueError("Cell lengths must be positive")
        a, b, c = float(a), float(b), float(c)
        rad = np.pi / 180.0  # f64::to_radians
        cos_alpha = float(np.cos(float(alpha) * rad))
        cos_beta = float(np.cos(float(beta) * rad))
        g = float(gamma) * rad
        sin_gamma, cos_gamma = float(np.sin(g)), float(np.cos(g))
        b_x = b * cos_gamma
        b_y = b * sin_gamma
        c_x = c * cos_beta
        c_y = c * (cos_alpha - cos_beta * cos_gamma) / sin_gamma
        c_z = float(np.sqrt(c * c - c_y * c_y - c_x * c_x))
        return cls([[a, b_x, c_x], [0.0, b_y, c_y], [0.0, 0.0, c_z]], cls.TRICLINIC)

    def matrix(self) -> np.ndarray:
        return np.array(self._m, dtype=np.float64)

    def inverse(self) -> np.ndarray:
        return np.array(self._inv, dtype=np.float64)

    def volume(self) -> float:
        """cells.rs:185-200."""
        m = self._m
        if self.shape == self.ORTHORHOMBIC:
            return m[0][0] * m[1][1] * m[2][2]
        va, vb, vc = ((m[0][k], m[1][k], m[2][k]) for k in range(3))
        return _dot(va, _cross(vb, vc))

    def fractional(self, v):
        return _mat_vec(self._inv, v)

    def cartesian(self, f):
        return _mat_vec(self._m, f)

    def scaled(self, factor: float) -> "UnitCell":
        """UnitCell::scale_mut(Matrix3::one() * factor) (cells.rs:201-207): the shape is kept."""
        f = float(factor)
        one = ((f * 1.0, f * 0.0, f * 0.0), (f * 0.0, f * 1.0, f * 0.0), (f * 0.0, f * 0.0, f * 1.0))
        return UnitCell(_mat_mul(self._m, one), self.shape)

    def wrap_vector(self, v):
        """cells.rs:263-282."""
        if self.shape == self.ORTHORHOMBIC:
            d = (self._m[0][0], self._m[1][1], self._m[2][2])
            return tuple(float(v[k]) - float(np.floor(float(v[k]) / d[k])) * d[k] for k in range(3))
        f = self.fractional(v)
        return self.cartesian(tuple(x - float(np.floor(x)) for x in f))

    def _lower(self):
        return np.ascontiguousarray(self.matrix().ravel()), (
            C.LG_CELL_ORTHORHOMBIC if self.shape == self.ORTHORHOMBIC else C.LG_CELL_TRICLINIC)


# ---------------------------------------------------------------------------
# Engine handle
# ---------------------------------------------------------------------------
class Engine:
    """Owns one lg_engine handle (a batch of `n_systems` systems)."""

    def __init__(self, n_systems: int = 1, precision: str = "fp64", skin: float = 1.0, device: int = 0,
                 threads_per_atom: int = 0, persistent: bool = True, cluster: int = 0, staging: bool = False):
        lib = C.load()
        prec = {"fp64": C.LG_PRECISION_FP64, "mixed": C.LG_PRECISION_MIXED}[precision]
        flags = 0 if persistent else C.LG_OPT_NO_PERSISTENT
        if staging:
            flags |= C.LG_OPT_STAGING
        if cluster:  # fixed cluster size of the persistent kernel (1, 2, 4 or 8)
            flags |= ({1: 1, 2: 2, 4: 3, 8: 4}[cluster]) << C.LG_OPT_CLUSTER_SHIFT
        opt = C.LgOptions(device, prec, skin, threads_per_atom, flags)
        handle = ctypes.c_void_p()
        C.check(lib.lg_create(ctypes.byref(opt), n_systems, ctypes.byref(handle)))
        self.lib = lib
        self.handle = handle
        self.n_systems = n_systems
        self.precision = precision

    def call(self, name: str, *args) -> None:
        C.check(getattr(self.lib, name)(self.handle, *args), self.handle)

    def run_steps(self, nsteps: int) -> int:
        """lg_md_run; returns the status (LG_ERR_NONFINITE still completes the
        steps of every system, see lg_system_status)."""
        return self.lib.lg_md_run(self.handle, int(nsteps))

    def check(self, code: int) -> None:
        C.check(code, self.handle)

    def close(self) -> None:
        if self.handle:
            self.lib.lg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, s: int, system: "System") -> None:
        """Lowers the description of `system` into system slot `s`."""
        system._lower_into(self, s)


# ---------------------------------------------------------------------------
# System
# ---------------------------------------------------------------------------
def _angles_from_bonds(bonds: list[tuple[int, int]]) -> list[tuple[int, int, int]]:
    """Angles of a bond set as Bonding::rebuild finds them (bonding.rs:78-110):
    every pair of distinct bonds sharing a particle j gives the angle (i, j, k)
    with i < k."""
    partners: dict[int, list[int]] = {}
    for a, b in bonds:
        partners.setdefault(a, []).append(b)
        partners.setdefault(b, []).append(a)
    angles = set()
    for j, ends in partners.items():
        for x in range(len(ends)):
            for y in range(x + 1, len(ends)):
                i, k = ends[x], ends[y]
                if i != k:
                    angles.add((min(i, k), j, max(i, k)))
    return sorted(angles)


def _dihedrals_from_bonds(bonds: list[tuple[int, int]]) -> list[tuple[int, int, int, int]]:
    """Dihedral angles of a bond set as Bonding::rebuild finds them
    (bonding.rs:111-157): every angle (i, j, k) with one more bond at an end
    gives a dihedral, oriented as Dihedral::new orders it (the end whose pair
    holds the smaller largest index first)."""
    def make(a, b, c, d):
        return (a, b, c, d) if max(a, b) < max(c, d) else (d, c, b, a)
    partners: dict[int, list[int]] = {}
    for a, b in bonds:
        partners.setdefault(a, []).append(b)
        partners.setdefault(b, []).append(a)
    out = set()
    for i, j, k in _angles_from_bonds(bonds):
        for q in partners.get(k, ()):  # a bond (k, q) other than (j, k)
            if q != j:
                out.add(make(i, j, k, q))
        for p in partners.get(i, ()):  # a bond (p, i) other than (i, j) and, in a 3-ring, (i, k)
            if p != j and p != k:
                out.add(make(p, i, j, k))
    return sorted(out)


class System:
    """Configuration + Interactions (lumol-core/src/sys/system.rs), evaluated on
    the GPU.  Particles of a molecule are contiguous, as in Lumol."""

    def __init__(self, cell: UnitCell, precision: str = "fp64", skin: float = 1.0):
        self.cell = cell
        self.precision = precision
        self.skin = skin
        self.names: list[str] = []
        self._kinds: dict[str, int] = {}
        self._pos: list = []
        self._charges: list[float] = []
        self._masses: list[float] = []
        self._mols: list[int] = []
        self._bonds: list[tuple[int, int]] = []
        self.velocities: np.ndarray | None = None
        self.pairs: dict[tuple[str, str], PairInteraction] = {}
        self.bond_potentials: dict[tuple[str, str], object] = {}
        self.angle_potentials: dict[tuple[str, str, str], object] = {}
        self.dihedral_potentials: dict[tuple[str, str, str, str], object] = {}
        self.coulomb = None
        self.step = 0
        # DegreesOfFreedom (sys/system.rs:18-26): "particles", "molecules" or
        # ("frozen", n); the device MD integrates every particle
        self.simulated_degrees_of_freedom = "particles"
        self.external_temperature: float | None = None
        self._engine: Engine | None = None
        self._positions = None
        self._version = 0
        self._uploaded = -1

    # ---- building ---------------------------------------------------------
    def _kind(self, name: str) -> int:
        if name not in self._kinds:
            self._kinds[name] = len(self._kinds)
        return self._kinds[name]

    def add_molecule(self, names, positions, bonds=(), charges=None, masses=None) -> int:
        """Adds one molecule; `bonds` index its particles from 0.  Returns the
        molecule index."""
        positions = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
        names = list(names)
        start = len(self.names)
        mol = (self._mols[-1] + 1) if self._mols else 0
        for a, name in enumerate(names):
            self._kind(name)
            self.names.append(name)
            self._charges.append(0.0 if charges is None else float(charges[a]))
            self._masses.append(ATOMIC_MASSES.get(name, 0.0) if masses is None else float(masses[a]))
            self._mols.append(mol)
        self._pos.append(positions)
        for i, j in bonds:
            self._bonds.append((start + min(i, j), start + max(i, j)))
        self._positions = None
        self._touch()
        return mol

    def add_particle(self, name: str, position, charge: float = 0.0, mass: float | None = None) -> None:
        self.add_molecule([name], [position], charges=[charge], masses=None if mass is None else [mass])

    def add_particles(self, names, positions, charges=None, masses=None) -> None:
        """Adds many single-particle molecules at once."""
        positions = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
        n = len(names)
        mol0 = (self._mols[-1] + 1) if self._mols else 0
        for a, name in enumerate(names):
            self._kind(name)
        self.names.extend(names)
        self._charges.extend([0.0] * n if charges is None else [float(q) for q in charges])
        self._masses.extend([ATOMIC_MASSES.get(nm, 0.0) for nm in names] if masses is None
                            else [float(m) for m in masses])
        self._mols.extend(range(mol0, mol0 + n))
        self._pos.append(positions)
        self._positions = None
        self._touch()

    def _touch(self) -> None:
        self._version += 1

    # ---- accessors ----------------------------------------------------------
    @property
    def size(self) -> int:
        return len(self.names)

    @property
    def positions(self) -> np.ndarray:
        if self._positions is None:
            self._positions = (np.ascontiguousarray(np.concatenate(self._pos, axis=0))
                               if self._pos else np.zeros((0, 3)))
            self._pos = [self._positions]
        return self._positions

    @positions.setter
    def positions(self, value) -> None:
        value = np.ascontiguousarray(value, dtype=np.float64).reshape(-1, 3)
        assert value.shape == (self.size, 3)
        self._positions = value
        self._pos = [value]

    @property
    def charges(self) -> np.ndarray:
        return np.array(self._charges, dtype=np.float64)

    def set_charge(self, i: int, q: float) -> None:
        self._charges[i] = float(q)
        self._touch()

    @property
    def masses(self) -> np.ndarray:
        return np.array(self._masses, dtype=np.float64)

    @property
    def kinds(self) -> np.ndarray:
        return np.array([self._kinds[nm] for nm in self.names], dtype=np.int32)

    @property
    def molecules(self) -> np.ndarray:
        return np.array(self._mols, dtype=np.int32)

    @property
    def bonds(self) -> list[tuple[int, int]]:
        return sorted(set(self._bonds))

    def angles(self) -> list[tuple[int, int, int]]:
        key = len(self._bonds)
        if getattr(self, "_angles_key", None) != key:
            self._angles_cache = _angles_from_bonds(self.bonds)
            self._angles_key = key
        return self._angles_cache

    def dihedrals(self) -> list[tuple[int, int, int, int]]:
        key = len(self._bonds)
        if getattr(self, "_dihedrals_key", None) != key:
            self._dihedrals_cache = _dihedrals_from_bonds(self.bonds)
            self._dihedrals_key = key
        return self._dihedrals_cache

    def molecule_range(self, molid: int) -> tuple[int, int]:
        mols = self.molecules
        idx = np.nonzero(mols == molid)[0]
        return int(idx[0]), int(idx[-1]) + 1

    def volume(self) -> float:
        return self.cell.volume()

    # ---- interactions -------------------------------------------------------
    def set_pair_potential(self, pair: tuple[str, str], interaction: PairInteraction) -> None:
        """System::set_pair_potential (sys/system.rs:122-131)."""
        if any(0.5 * d < interaction.cutoff for d in self.cell.lengths):
            raise ValueError(
                "Can not add a potential with a cutoff bigger than half of the smallest cell length. "
                "Try increasing the cell size or decreasing the cutoff."
            )
        self._kind(pair[0])
        self._kind(pair[1])
        self.pairs[tuple(sorted(pair))] = interaction
        self._touch()

    def set_bond_potential(self, pair: tuple[str, str], potential) -> None:
        self.bond_potentials[tuple(sorted(pair))] = potential
        self._touch()

    def set_angle_potential(self, angle: tuple[str, str, str], potential) -> None:
        a, b, c = angle
        self.angle_potentials[(min(a, c), b, max(a, c))] = potential
        self._touch()

    def set_dihedral_potential(self, dihedral: tuple[str, str, str, str], potential) -> None:
        """System::set_dihedral_potential: the potential of the dihedral angles
        whose particles have these names, in either direction."""
        self.dihedral_potentials[min(tuple(dihedral), tuple(reversed(dihedral)))] = potential
        self._touch()

    def dihedral_potential(self, names: tuple[str, str, str, str]):
        return self.dihedral_potentials.get(min(tuple(names), tuple(reversed(names))))

    def set_coulomb_potential(self, potential) -> None:
        """System::set_coulomb_potential (sys/system.rs:159-170)."""
        if any(0.5 * d < potential.cutoff for d in self.cell.lengths):
            raise ValueError(
                "Can not add a potential with a cutoff bigger than half of the smallest cell length. "
                "Try increasing the cell size or decreasing the cutoff."
            )
        self.coulomb = potential
        self._touch()

    # ---- lowering ---------------------------------------------------------------
    def pair_table(self) -> list:
        names = sorted(self._kinds, key=self._kinds.get)
        nk = len(names)
        table = (C.LgPair * (nk * nk))()
        for a, na in enumerate(names):
            for b, nb in enumerate(names):
                inter = self.pairs.get(tuple(sorted((na, nb))))
                table[a * nk + b] = inter._lower() if inter else C.LgPair()
        return nk, table

    def _bonded(self, pot) -> C.LgBonded:
        if pot is None:
            return C.LgBonded(C.LG_PAIR_ABSENT, 0, 0.0, 0.0, 0.0)
        kind, par = pot._params()
        if kind == C.LG_PAIR_MORSE:  # Morse {a, x0, depth}
            return C.LgBonded(kind, 0, par[2], par[1], par[0])
        k, x0, extra = par
        return C.LgBonded(kind, int(extra) if kind == C.LG_BONDED_TORSION else 0, k, x0, 0.0)

    def _lower_into(self, eng: Engine, s: int) -> None:
        n = self.size
        m, shape = self.cell._lower()
        eng.call("lg_set_cell_ex", s, C.dptr(m), shape)
        kinds = self.kinds
        charges = self.charges
        masses = self.masses
        mols = self.molecules
        eng.call("lg_set_particles", s, n, C.iptr(kinds), C.dptr(charges), C.dptr(masses), C.iptr(mols))
        nk, table = self.pair_table()
        eng.call("lg_set_pairs", s, nk, table)
        bonds = self.bonds
        barr = np.array(bonds, dtype=np.int32).reshape(-1)
        bpots = (C.LgBonded * max(len(bonds), 1))()
        for b, (i, j) in enumerate(bonds):
            bpots[b] = self._bonded(self.bond_potentials.get(tuple(sorted((self.names[i], self.names[j])))))
        eng.call("lg_set_bonds", s, len(bonds), C.iptr(barr), bpots)
        angles = self.angles()
        aarr = np.array(angles, dtype=np.int32).reshape(-1)
        apots = (C.LgBonded * max(len(angles), 1))()
        for a, (i, j, k) in enumerate(angles):
            ni, nj, nk_ = self.names[i], self.names[j], self.names[k]
            apots[a] = self._bonded(self.angle_potentials.get((min(ni, nk_), nj, max(ni, nk_))))
        eng.call("lg_set_angles", s, len(angles), C.iptr(aarr), apots)
        dihedrals = self.dihedrals()
        darr = np.array(dihedrals, dtype=np.int32).reshape(-1)
        dpots = (C.LgBonded * max(len(dihedrals), 1))()
        for d, q in enumerate(dihedrals):
            dpots[d] = self._bonded(self.dihedral_potential(tuple(self.names[x] for x in q)))
        eng.call("lg_set_dihedrals", s, len(dihedrals), C.iptr(darr), dpots)
        coul = self.coulomb._lower() if self.coulomb is not None else C.LgCoulomb()
        eng.call("lg_set_coulomb", s, ctypes.byref(coul))

    def engine(self) -> Engine:
        if self._engine is None:
            self._engine = Engine(1, self.precision, self.skin)
        if self._uploaded != self._version:
            self._lower_into(self._engine, 0)
            self._uploaded = self._version
        return self._engine

    # ---- computations -------------------------------------------------------------
    def compute(self, terms: int = C.LG_TERM_ALL, want: int = 7):
        """Forces, energy and virial of the requested terms in one GPU pass."""
        eng = self.engine()
        pos = np.ascontiguousarray(self.positions, dtype=np.float64)
        forces = np.zeros((self.size, 3))
        energy = ctypes.c_double(0.0)
        virial = np.zeros(9)
        eng.call("lg_compute", 0, C.dptr(pos), terms, want, C.dptr(forces), ctypes.byref(energy),
                 C.dptr(virial))
        return forces, energy.value, virial.reshape(3, 3)

    def forces(self) -> np.ndarray:
        """System::forces (sys/system.rs:316-318)."""
        return self.compute(C.LG_TERM_ALL, C.LG_WANT_FORCES)[0]

    def potential_energy(self) -> float:
        """System::potential_energy (sys/system.rs:263-265)."""
        return self.compute(C.LG_TERM_ALL, C.LG_WANT_ENERGY)[1]

    def atomic_virial(self) -> np.ndarray:
        """AtomicVirial::compute (sys/compute.rs:195-254)."""
        return self.compute(C.LG_TERM_ALL, C.LG_WANT_VIRIAL)[2]

    def virial(self) -> np.ndarray:
        """System::virial / Virial::compute (sys/compute.rs:372-380): the
        molecular definition when the simulated degrees of freedom are the
        molecules', else the atomic one."""
        if self.simulated_degrees_of_freedom == "molecules":
            return self.molecular_virial()
        return self.atomic_virial()

    def degrees_of_freedom(self) -> int:
        """System::degrees_of_freedom (sys/system.rs:249-255)."""
        dof = self.simulated_degrees_of_freedom
        if dof == "particles":
            return 3 * self.size
        if dof == "molecules":
            return 3 * len(set(self._mols))
        return 3 * self.size - int(dof[1])  # ("frozen", n)

    def pressure_at_temperature(self, temperature: float) -> float:
        """PressureAtTemperature (sys/compute.rs:383-397)."""
        from .units import K_BOLTZMANN
        if not temperature >= 0.0:
            raise ValueError("the temperature must be positive")
        virial = float(np.trace(self.virial()))
        return (self.degrees_of_freedom() * K_BOLTZMANN * temperature + virial) / (3.0 * self.volume())

    def pressure(self) -> float:
        """Pressure (sys/compute.rs:403-410), at the kinetic temperature."""
        return self.pressure_at_temperature(self.temperature())

    def stress_at_temperature(self, temperature: float) -> np.ndarray:
        """StressAtTemperature (sys/compute.rs:418-433)."""
        from .units import K_BOLTZMANN
        if not temperature >= 0.0:
            raise ValueError("the temperature must be positive")
        kinetic = self.degrees_of_freedom() / 3.0 * K_BOLTZMANN * temperature * np.eye(3)
        return (kinetic + self.virial()) / self.volume()

    def stress(self) -> np.ndarray:
        """Stress (sys/compute.rs:436-445), at the kinetic temperature."""
        return self.stress_at_temperature(self.temperature())

    def molecular_virial(self, terms: int = C.LG_TERM_ALL) -> np.ndarray:
        """MolecularVirial::compute (sys/compute.rs:278-362): the virial with
        the molecular definition (FP64 systems)."""
        eng = self.engine()
        pos = np.ascontiguousarray(self.positions, dtype=np.float64)
        virial = np.zeros(9)
        eng.call("lg_molecular_virial", 0, C.dptr(pos), terms, C.dptr(virial))
        return virial.reshape(3, 3)

    def energy_term(self, terms: int) -> float:
        return self.compute(terms, C.LG_WANT_ENERGY)[1]

    def pair_set(self, family: int = 0) -> np.ndarray:
        """(i, j) pairs, i < j, that the device counts for a family
        (0: pair potentials, 1: real-space Coulomb), sorted."""
        eng = self.engine()
        pos = np.ascontiguousarray(self.positions, dtype=np.float64)
        count = ctypes.c_int64(0)
        cap = 1 << 16
        while True:
            out = np.zeros(2 * cap, dtype=np.int32)
            eng.call("lg_pairset", 0, C.dptr(pos), family, C.iptr(out), cap, ctypes.byref(count))
            if count.value <= cap:
                return out[: 2 * count.value].reshape(-1, 2)
            cap = int(count.value)

    # ---- Monte Carlo (EnergyCache, sys/cache.rs) -----------------------------------------
    def mc_init(self) -> float:
        """EnergyCache::init (cache.rs:75-98): returns the cached total energy."""
        eng = self.engine()
        pos = np.ascontiguousarray(self.positions, dtype=np.float64)
        energy = ctypes.c_double(0.0)
        eng.call("lg_mc_init", 0, C.dptr(pos), ctypes.byref(energy))
        return energy.value

    def move_molecule_cost(self, molid: int, new_positions) -> float:
        """EnergyCache::move_molecule_cost (cache.rs:145-220): energy change of
        moving molecule `molid` to `new_positions`."""
        newpos = np.ascontiguousarray(new_positions, dtype=np.float64)
        cost = ctypes.c_double(0.0)
        self.engine().call("lg_mc_move_molecule_cost", 0, molid, C.dptr(newpos), ctypes.byref(cost))
        return cost.value

    def mc_update(self, molid: int, molecule_positions) -> float:
        """EnergyCache::update (cache.rs:118-127) after the move was applied;
        returns the new cached energy."""
        newpos = np.ascontiguousarray(molecule_positions, dtype=np.float64)
        energy = ctypes.c_double(0.0)
        self.engine().call("lg_mc_update", 0, C.dptr(newpos), ctypes.byref(energy))
        lo, hi = self.molecule_range(molid)
        pos = self.positions.copy()
        pos[lo:hi] = newpos.reshape(-1, 3)
        self.positions = pos
        return energy.value

    def wrap_molecule(self, molid: int, positions) -> np.ndarray:
        """Molecule::wrap (sys/config/molecules.rs:287-296): shift the molecule so
        that its centre of mass lies in the cell (UnitCell::wrap_vector)."""
        lo, hi = self.molecule_range(molid)
        m = self.masses[lo:hi]
        positions = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
        total = 0.0
        com = np.zeros(3)
        for a in range(hi - lo):
            total += m[a]
            com = com + m[a] * positions[a]
        com = com / total
        wrapped = np.array(self.cell.wrap_vector(com))
        return positions + (wrapped - com)

    def kinetic_energy(self) -> float:
        v = self.velocities
        return float(sum(0.5 * m * float(np.dot(vi, vi)) for m, vi in zip(self._masses, v)))

    def simulated_temperature(self, temperature: float | None) -> None:
        """System::simulated_temperature (sys/system.rs): an external
        temperature that temperature() returns instead of the kinetic one."""
        if temperature is not None and not temperature >= 0.0:
            raise ValueError("the temperature must be positive")
        self.external_temperature = temperature

    def temperature(self) -> float:
        """System::temperature (sys/system.rs:273-278): the external
        temperature if one is set, else Temperature (sys/compute.rs:165-172),
        2 K / (dof k_B)."""
        from .units import K_BOLTZMANN
        if self.external_temperature is not None:
            return self.external_temperature
        return 2.0 * self.kinetic_energy() / (self.degrees_of_freedom() * K_BOLTZMANN)


# ---------------------------------------------------------------------------
# Molecular dynamics (lumol-sim/src/md)
# ---------------------------------------------------------------------------
@dataclass
class VelocityVerlet:
    """VelocityVerlet::new(timestep) (md/integrators.rs:19-70)."""
    timestep: float
    _kind = C.LG_INTEGRATOR_VELOCITY_VERLET


@dataclass
class BerendsenBarostat:
    """BerendsenBarostat::new(timestep, pressure, tau) (md/integrators.rs:174-250):
    Velocity-Verlet with the positions scaled by eta and the cell by eta^3 at
    every step, eta^3 = 1 - 7372 / tau (pressure - P) from the pressure of the
    previous step.  The cell changes on the device; MolecularDynamics.run
    brings the new cell back into System.cell."""
    timestep: float
    pressure: float
    tau: float
    _kind = C.LG_INTEGRATOR_VELOCITY_VERLET


class AnisoBerendsenBarostat:
    """AnisoBerendsenBarostat::new(timestep, stress, tau) (md/integrators.rs:252-342):
    Velocity-Verlet with the positions scaled by the matrix eta (x = eta x) and
    the cell by it (cell * eta, shape kept) at every step, eta = 1 - dt 7372 /
    tau (stress - Stress) made symmetric, from the stress tensor of the
    previous step.  `hydrostatic(timestep, pressure, tau)` takes stress =
    pressure * 1."""
    _kind = C.LG_INTEGRATOR_VELOCITY_VERLET

    def __init__(self, timestep: float, stress, tau: float):
        self.timestep = float(timestep)
        self.stress = np.asarray(stress, dtype=np.float64).reshape(3, 3).copy()
        self.tau = float(tau)

    @classmethod
    def hydrostatic(cls, timestep: float, pressure: float, tau: float) -> "AnisoBerendsenBarostat":
        return cls(timestep, float(pressure) * np.eye(3), tau)


@dataclass
class Verlet:
    """Verlet::new(timestep) (md/integrators.rs:72-123): keeps the positions at
    t - dt, taken as x - v dt at setup."""
    timestep: float
    _kind = C.LG_INTEGRATOR_VERLET


@dataclass
class LeapFrog:
    """LeapFrog::new(timestep) (md/integrators.rs:125-169)."""
    timestep: float
    _kind = C.LG_INTEGRATOR_LEAP_FROG


def _check_temperature(temperature: float) -> None:
    if temperature < 0.0:
        raise ValueError("The temperature must be positive in thermostats.")


@dataclass
class BerendsenThermostat:
    """BerendsenThermostat::new(temperature, tau) (md/thermostats.rs:77-121)."""
    temperature: float
    tau: float

    def __post_init__(self):
        _check_temperature(self.temperature)
        if self.tau < 1.0:
            raise ValueError("The timestep must be larger than 1 in berendsen thermostat.")

    def _params(self, p) -> None:
        p.thermostat, p.temperature, p.tau = C.LG_THERMOSTAT_BERENDSEN, self.temperature, self.tau


@dataclass
class RescaleThermostat:
    """RescaleThermostat::new(temperature) / with_tolerance(temperature, tol)
    (md/thermostats.rs:27-73): velocities rescaled to `temperature` when the
    instant temperature is further than `tolerance` from it (default 5 %)."""
    temperature: float
    tolerance: float | None = None

    def __post_init__(self):
        _check_temperature(self.temperature)
        if self.tolerance is None:
            self.tolerance = 0.05 * self.temperature

    def _params(self, p) -> None:
        p.thermostat, p.temperature, p.tolerance = C.LG_THERMOSTAT_RESCALE, self.temperature, self.tolerance


@dataclass
class CSVRThermostat:
    """CSVRThermostat::new(temperature, tau) (md/thermostats.rs:123-210).  The
    noise comes from SplitMix64 streams of (seed, application count) instead of
    the reference's xorshift generator: the same distribution, other numbers."""
    temperature: float
    tau: float
    seed: int = 0

    def __post_init__(self):
        _check_temperature(self.temperature)
        if self.tau < 1.0:
            raise ValueError("The timestep must be larger than 1 in CSVR thermostat.")

    def _params(self, p) -> None:
        p.thermostat, p.temperature, p.tau = C.LG_THERMOSTAT_CSVR, self.temperature, self.tau
        p.seed = self.seed & (2 ** 64 - 1)


class RemoveTranslation:
    """RemoveTranslation control (md/controls.rs:26-43)."""
    _bit = C.LG_CONTROL_REMOVE_TRANSLATION


class RemoveRotation:
    """RemoveRotation control (md/controls.rs:44-71)."""
    _bit = C.LG_CONTROL_REMOVE_ROTATION


class Rewrap:
    """Rewrap control (md/controls.rs:73-89): molecules' centres of mass back into the cell."""
    _bit = C.LG_CONTROL_REWRAP


def md_params(integrator, thermostat=None, controls=()) -> "C.LgMdParams":
    """The C ABI's lg_md_params for an integrator, an optional thermostat and controls."""
    p = C.LgMdParams()
    p.integrator = integrator._kind
    p.timestep = integrator.timestep
    if thermostat is not None:
        thermostat._params(p)
    for c in controls:
        p.controls |= c._bit
    return p


@dataclass
class MolecularDynamics:
    """MolecularDynamics propagator (md/molecular_dynamics.rs:11-83): integrate,
    then thermostat, then controls, every step, with the state resident on the GPU."""
    integrator: VelocityVerlet | Verlet | LeapFrog
    thermostat: BerendsenThermostat | RescaleThermostat | CSVRThermostat | None = None
    controls: tuple = ()
    _ready: bool = field(default=False, repr=False)

    def setup(self, system: System) -> None:
        """Propagator::setup: the integrator's setup (accelerations := 0, or
        Verlet's positions at t - dt) at the first run."""
        # Simulation::run (lumol-sim/src/simulations.rs:70-86): MD takes the
        # temperature from the velocities and moves every particle
        system.simulated_temperature(None)
        system.simulated_degrees_of_freedom = "particles"
        eng = system.engine()
        p = md_params(self.integrator, self.thermostat, self.controls)
        eng.call("lg_md_setup_ex", 0, ctypes.byref(p))
        if isinstance(self.integrator, BerendsenBarostat):
            eng.call("lg_md_set_barostat", 0, C.LG_BAROSTAT_BERENDSEN, float(self.integrator.pressure),
                     float(self.integrator.tau))
        elif isinstance(self.integrator, AnisoBerendsenBarostat):
            stress = np.ascontiguousarray(self.integrator.stress.ravel())
            eng.call("lg_md_set_aniso_barostat", 0, C.dptr(stress), float(self.integrator.tau))
        if system.velocities is None:
            system.velocities = np.zeros((system.size, 3))
        pos = np.ascontiguousarray(system.positions)
        vel = np.ascontiguousarray(system.velocities, dtype=np.float64)
        eng.call("lg_md_set_state", 0, C.dptr(pos), C.dptr(vel))
        self._ready = True

    def run(self, system: System, nsteps: int) -> None:
        """`nsteps` calls of Propagator::propagate, then the state is read back."""
        if not self._ready:
            self.setup(system)
        eng = system.engine()
        eng.call("lg_md_run", int(nsteps))
        pos = np.zeros((system.size, 3))
        vel = np.zeros((system.size, 3))
        eng.call("lg_md_get_state", 0, C.dptr(pos), C.dptr(vel))
        system.positions = pos
        system.velocities = vel
        system.step += int(nsteps)
        if isinstance(self.integrator, (BerendsenBarostat, AnisoBerendsenBarostat)):  # the cell the barostat left
            m = np.zeros(9)
            eng.call("lg_get_cell", 0, C.dptr(m))
            system.cell = UnitCell(m.reshape(3, 3), system.cell.shape)
            system._uploaded = system._version  # the engine already holds this cell


# ---------------------------------------------------------------------------
# Monte Carlo (lumol-sim/src/mc)
# ---------------------------------------------------------------------------
class Translate:
    """Translate move (mc/moves/translate.rs:20-125): a uniform displacement in
    [-delta / sqrt(3), delta / sqrt(3)) per axis of one random molecule."""

    def __init__(self, delta: float):
        if not delta > 0.0:
            raise ValueError("delta must be positive in Translate move")
        self.delta = delta / np.sqrt(3.0)


class Rotate:
    """Rotate move (mc/moves/rotate.rs:24-125): one random molecule rotated
    about its centre of mass by an angle uniform in [-theta, theta) around an
    axis uniform on the unit sphere (Matrix3::rotation, types/matrix.rs:149-176)."""

    def __init__(self, theta: float):
        if not theta > 0.0:
            raise ValueError("theta must be positive in Rotate move")
        self.theta = float(theta)


class Resize:
    """Resize move (mc/moves/resize.rs:14-128) for NPT Monte Carlo: the volume
    changes by a uniform delta in [-delta, delta), the cell is scaled by
    cbrt((V + delta) / V) and every molecule moves with its centre of mass
    (fractional coordinates kept); the cost is
    beta (dE + P dV) - N_molecules ln(V' / V), dE from
    EnergyCache::move_all_molecules_cost on the GPU."""

    def __init__(self, pressure: float, delta: float):
        if not delta > 0.0:
            raise ValueError("delta must be positive in Resize move")
        self.pressure = float(pressure)
        self.delta = float(delta)


def _ortho_inverse(L) -> np.ndarray:
    """The diagonal of Matrix3::inverse of diag(a, b, c) (types/matrix.rs:212-227)."""
    a, b, c = (float(x) for x in L)
    det = a * (b * c - 0.0 * 0.0) - 0.0 * (0.0 * c - 0.0 * 0.0) + 0.0 * (0.0 * 0.0 - b * 0.0)
    inv = 1.0 / det
    return np.array([(b * c - 0.0 * 0.0) * inv, (a * c - 0.0 * 0.0) * inv, (a * b - 0.0 * 0.0) * inv])


def _rotation(axis: np.ndarray, angle: float) -> np.ndarray:
    """Matrix3::rotation (types/matrix.rs:149-169) around `axis` (normalised):
    the matrix with the reference's sign convention, which turns e3 into e2
    for a quarter turn around e1."""
    n = axis / np.sqrt(axis @ axis)
    c, s_ = np.cos(angle), np.sin(angle)
    t = 1.0 - c
    xs, ys, zs = n * s_
    xy, xz, yz = n[0] * n[1] * t, n[0] * n[2] * t, n[1] * n[2] * t
    return np.array([[n[0] * n[0] * t + c, xy + zs, xz - ys],
                     [xy - zs, n[1] * n[1] * t + c, yz + xs],
                     [xz + ys, yz - xs, n[2] * n[2] * t + c]])


class MonteCarlo:
    """Metropolis propagator (mc/monte_carlo.rs:289-329) with Translate and
    Rotate moves, each picked with its frequency (MonteCarlo::add); the move
    costs run on the GPU.  The random stream is numpy's, seeded (the
    reference's xorshift stream is not reproduced)."""

    def __init__(self, temperature: float, move, seed: int = 0):
        """`move`: a Translate or Rotate, or a list of (move, frequency)."""
        from .units import K_BOLTZMANN
        self.temperature = float(temperature)
        self.beta = 1.0 / (K_BOLTZMANN * temperature)
        moves = [(move, 1.0)] if isinstance(move, (Translate, Rotate, Resize)) else [(m, float(f)) for m, f in move]
        if not moves or any(not f > 0.0 for _, f in moves):
            raise ValueError("MonteCarlo needs moves with positive frequencies")
        self.moves = [m for m, _ in moves]
        freq = np.array([f for _, f in moves])
        self.frequencies = freq / freq.sum()
        self.move = self.moves[0]
        self.rng = np.random.default_rng(seed)
        self.accepted = 0
        self.attempted = 0
        self.energy = None

    def setup(self, system: System) -> None:
        # Simulation::run (lumol-sim/src/simulations.rs:70-86) with MonteCarlo's
        # temperature strategy and degrees of freedom (mc/monte_carlo.rs:243-279):
        # the external temperature, and rigid molecules for Translate
        system.simulated_temperature(self.temperature)
        system.simulated_degrees_of_freedom = "molecules"
        self.energy = system.mc_init()

    def _resize(self, system: System, move: Resize) -> None:
        """Resize::prepare / cost / apply / restore (resize.rs:63-124)."""
        eng = system.engine()
        old = system.cell
        volume = old.volume()
        delta = self.rng.uniform(-move.delta, move.delta)
        scaling = float(np.cbrt((volume + delta) / volume))
        new = old.scaled(scaling)  # UnitCell::scale_mut(Matrix3::one() * scaling)
        pos = system.positions
        newpos = pos.copy()
        m = system.masses
        for mol in range(int(system.molecules[-1]) + 1):
            lo, hi = system.molecule_range(mol)
            total, com = 0.0, np.zeros(3)
            for a in range(lo, hi):  # Molecule::center_of_mass (molecules.rs:256-264)
                total += m[a]
                com = com + m[a] * pos[a]
            com = com / total
            frac = old.fractional(com)  # previous.cell.fractional(com)
            delta_com = np.array(new.cartesian(frac)) - com  # cell.cartesian(frac) - com
            newpos[lo:hi] = pos[lo:hi] + delta_com
        cell = np.ascontiguousarray(new.matrix().ravel())
        de = ctypes.c_double(0.0)
        eng.call("lg_mc_move_all_molecules_cost", 0, C.dptr(cell), C.dptr(np.ascontiguousarray(newpos)),
                 ctypes.byref(de))
        new_volume = new.volume()
        nmol = int(system.molecules[-1]) + 1
        cost = self.beta * (de.value + move.pressure * (new_volume - volume)) - nmol * np.log(new_volume / volume)
        self.attempted += 1
        if cost <= 0.0 or self.rng.random() < np.exp(-cost):
            energy = ctypes.c_double(0.0)
            eng.call("lg_mc_update", 0, None, ctypes.byref(energy))
            self.energy = energy.value
            system.cell = new
            system.positions = newpos
            system._uploaded = system._version  # the engine holds the new cell and positions
            self.accepted += 1
        else:
            eng.call("lg_mc_restore", 0)

    def propagate(self, system: System) -> None:
        nmol = int(system.molecules[-1]) + 1
        move = self.moves[int(self.rng.choice(len(self.moves), p=self.frequencies))] if len(self.moves) > 1 \
            else self.moves[0]
        if isinstance(move, Resize):
            self._resize(system, move)
            return
        molid = int(self.rng.integers(nmol))
        lo, hi = system.molecule_range(molid)
        if isinstance(move, Rotate):
            pos = system.positions[lo:hi]
            m = system.masses[lo:hi, None]
            com = (m * pos).sum(axis=0) / m.sum()
            axis = self.rng.normal(size=3)
            rot = _rotation(axis, self.rng.uniform(-move.theta, move.theta))
            newpos = com + (pos - com) @ rot.T
        else:
            delta = self.rng.uniform(-move.delta, move.delta, size=3)
            newpos = system.positions[lo:hi] + delta
        cost = self.beta * system.move_molecule_cost(molid, newpos)
        self.attempted += 1
        if cost <= 0.0 or self.rng.random() < np.exp(-cost):
            # Translate::apply wraps the molecule's centre of mass into the cell
            # (translate.rs:114-125); Rotate::apply only copies the new positions
            # (rotate.rs:91-96)
            if isinstance(move, Translate):
                newpos = system.wrap_molecule(molid, newpos)
            self.energy = system.mc_update(molid, newpos)
            self.accepted += 1
