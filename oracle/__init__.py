"""CPU oracle of the parity tests -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper around `lumol_oracle.cpp`, a C++17 restatement of
lumol-core's CPU arithmetic (see the header of that file for the files it
follows).  Only the tests, `__graft_entry__.smoke()` and bench.py's CPU
baseline use it, as the checker; the engine never imports it.

Parity pin: tests/test_oracle_reference.py checks this oracle against the
reference's own unit-test literals and its NIST LJ / SPC/E data.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "lumol_oracle.cpp")
LIB = os.path.join(HERE, "_build", "liblumol_oracle.so")

TERM_PAIRS, TERM_TAIL, TERM_BONDS, TERM_ANGLES = 1, 2, 4, 8
TERM_COUL_REAL, TERM_COUL_SELF, TERM_COUL_KSPACE, TERM_DIHEDRALS, TERM_ALL = 16, 32, 64, 128, 255


def build(force: bool = False) -> str:
    """Compiles the oracle with g++ (-ffp-contract=off: Rust never fuses a*b+c)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    hdr = os.path.join(HERE, "lumol_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-o", tmp, SRC]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout + proc.stderr)
    os.replace(tmp, LIB)
    return LIB


class OrcPair(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("shifted", ctypes.c_int32), ("restriction", ctypes.c_int32),
                ("tail", ctypes.c_int32), ("p0", ctypes.c_double), ("p1", ctypes.c_double),
                ("p2", ctypes.c_double), ("cutoff", ctypes.c_double), ("scale14", ctypes.c_double),
                ("p3", ctypes.c_double), ("p4", ctypes.c_double), ("table_size", ctypes.c_int32),
                ("table_pad", ctypes.c_int32), ("table_max", ctypes.c_double)]


class OrcBonded(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("n", ctypes.c_int32), ("k", ctypes.c_double), ("x0", ctypes.c_double),
                ("a", ctypes.c_double)]


class OrcCoulomb(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("restriction", ctypes.c_int32), ("kmax", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("cutoff", ctypes.c_double), ("alpha", ctypes.c_double),
                ("scale14", ctypes.c_double)]


class OrcDesc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("positions", ctypes.c_void_p), ("kinds", ctypes.c_void_p),
                ("charges", ctypes.c_void_p), ("masses", ctypes.c_void_p), ("molecules", ctypes.c_void_p),
                ("n_bonds", ctypes.c_int64), ("bonds", ctypes.c_void_p), ("n_kinds", ctypes.c_int32),
                ("pairs", ctypes.POINTER(OrcPair)), ("bond_pots", ctypes.POINTER(OrcBonded)),
                ("angle_pots", ctypes.POINTER(OrcBonded)), ("coulomb", OrcCoulomb),
                ("cell", ctypes.c_double * 3), ("dihedral_pots", ctypes.POINTER(OrcBonded)),
                ("cell_shape", ctypes.c_int32), ("cell_pad", ctypes.c_int32), ("cell_matrix", ctypes.c_double * 9)]

CELL_ORTHORHOMBIC, CELL_TRICLINIC = 0, 1


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        P, D, V = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [ctypes.POINTER(OrcDesc)]
        lib.orc_destroy.argtypes = [P]
        lib.orc_num_threads.restype = ctypes.c_int
        lib.orc_set_threads.argtypes = [ctypes.c_int]
        lib.orc_set_positions.argtypes = [P, V]
        lib.orc_get_positions.argtypes = [P, V]
        lib.orc_n_angles.restype = ctypes.c_int64
        lib.orc_n_angles.argtypes = [P]
        lib.orc_angles.argtypes = [P, V]
        lib.orc_energy.restype = ctypes.c_double
        lib.orc_energy.argtypes = [P, ctypes.c_int]
        lib.orc_forces.argtypes = [P, ctypes.c_int, V]
        lib.orc_virial.argtypes = [P, ctypes.c_int, V]
        lib.orc_molecular_virial.argtypes = [P, ctypes.c_int, V]
        lib.orc_pairset.restype = ctypes.c_int64
        lib.orc_pairset.argtypes = [P, ctypes.c_int, V, ctypes.c_int64]
        lib.orc_velocity_verlet.argtypes = [P, V, V, V, ctypes.c_double, ctypes.c_int64, ctypes.c_double,
                                            ctypes.c_double]
        lib.orc_md_run.argtypes = [P, V, V, V, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                   ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32, ctypes.c_int64]
        lib.orc_verlet_setup.argtypes = [P, V, V, ctypes.c_double, V]
        lib.orc_temperature.restype = ctypes.c_double
        lib.orc_temperature.argtypes = [P, V]
        lib.orc_kinetic_energy.restype = ctypes.c_double
        lib.orc_kinetic_energy.argtypes = [P, V]
        lib.orc_set_cell.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.orc_get_cell.argtypes = [P, V]
        lib.orc_set_cell_matrix.argtypes = [P, V, ctypes.c_int32]
        lib.orc_get_cell_matrix.argtypes = [P, V]
        lib.orc_cell_info.argtypes = [P, V, V]
        lib.orc_cell_apply.argtypes = [P, V, ctypes.c_int32]
        lib.orc_aniso_barostat_run.restype = ctypes.c_int
        lib.orc_aniso_barostat_run.argtypes = [P, V, V, V, V, ctypes.c_double, V, ctypes.c_double, ctypes.c_int64]
        lib.orc_maximum_cutoff.restype = ctypes.c_double
        lib.orc_maximum_cutoff.argtypes = [P]
        lib.orc_berendsen_barostat_run.restype = ctypes.c_int
        lib.orc_berendsen_barostat_run.argtypes = [P, V, V, V, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_int64]
        lib.orc_move_all_molecules_cost.restype = ctypes.c_double
        lib.orc_move_all_molecules_cost.argtypes = [P, V, V]
        lib.orc_cache_restore.argtypes = [P]
        lib.orc_cache_init.argtypes = [P]
        lib.orc_cache_energy.restype = ctypes.c_double
        lib.orc_cache_energy.argtypes = [P]
        lib.orc_move_molecule_cost.restype = ctypes.c_double
        lib.orc_move_molecule_cost.argtypes = [P, ctypes.c_int64, V]
        lib.orc_cache_update.argtypes = [P]
        lib.orc_pair_eval.argtypes = [ctypes.POINTER(OrcPair), ctypes.c_double, D, D, D, D]
        lib.orc_bonded_eval.argtypes = [ctypes.POINTER(OrcBonded), ctypes.c_double, D, D]
        lib.orc_dihedral_geometry.argtypes = [V, V, V, V, V, D, V]
        lib.orc_n_dihedrals.restype = ctypes.c_int64
        lib.orc_n_dihedrals.argtypes = [P]
        lib.orc_dihedrals.argtypes = [P, V]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _state_array(a, n: int, copy: bool = False) -> np.ndarray:
    """An (n, 3) float64 C-contiguous copy or view of a state array; anything
    else (None, a wrong shape) is an error, since the library reads and writes
    3 n doubles through the pointer."""
    if a is None:
        raise ValueError("state array is None")
    arr = np.ascontiguousarray(a, dtype=np.float64)
    if arr.size != 3 * n:
        raise ValueError(f"state array has {arr.size} values, expected {3 * n}")
    return arr.copy() if copy else arr


class Oracle:
    """Oracle restatement of one Lumol System.

    `spec` is any object with the attributes of a lumol_gb300.System
    (positions, kinds, charges, masses, molecules, bonds, names, pairs,
    bond_potentials, angle_potentials, coulomb, cell, _kinds)."""

    def __init__(self, spec):
        lib = load()
        self.lib = lib
        names = sorted(spec._kinds, key=spec._kinds.get)
        nk = len(names)
        self.n = spec.size
        self._keep = []

        def keep(a):
            a = np.ascontiguousarray(a)
            self._keep.append(a)
            return a

        pos = keep(np.asarray(spec.positions, dtype=np.float64))
        kinds = keep(np.asarray(spec.kinds, dtype=np.int32))
        charges = keep(np.asarray(spec.charges, dtype=np.float64))
        masses = keep(np.asarray(spec.masses, dtype=np.float64))
        mols = keep(np.asarray(spec.molecules, dtype=np.int32))
        bonds = keep(np.array(spec.bonds, dtype=np.int32).reshape(-1))
        pairs = (OrcPair * (nk * nk))()
        bpots = (OrcBonded * (nk * nk))()
        apots = (OrcBonded * (nk * nk * nk))()
        dpots = (OrcBonded * (nk * nk * nk * nk))()
        for a, na in enumerate(names):
            for b, nb in enumerate(names):
                inter = spec.pairs.get(tuple(sorted((na, nb))))
                if inter is not None:
                    kind, params = inter.potential._params()
                    p0, p1, p2, p3, p4 = (list(params) + [0.0] * 5)[:5]
                    r = inter.restriction
                    rr, s14 = (r[0], r[1]) if isinstance(r, tuple) else (r, 1.0)
                    tsize, tmax = getattr(inter.potential, "_table", (0, 0.0))
                    pairs[a * nk + b] = OrcPair(kind, int(inter.shifted_energy), rr, int(inter.tail),
                                                p0, p1, p2, inter.cutoff, s14, p3, p4, tsize, 0, tmax)
                bp = spec.bond_potentials.get(tuple(sorted((na, nb))))
                if bp is not None:
                    bpots[a * nk + b] = _orc_bonded(bp)
                for c, nc in enumerate(names):
                    ap = spec.angle_potentials.get((min(na, nc), nb, max(na, nc)))
                    if ap is not None:
                        apots[(a * nk + b) * nk + c] = _orc_bonded(ap)
                    for d, nd in enumerate(names):
                        dp = spec.dihedral_potential((na, nb, nc, nd))
                        if dp is not None:
                            dpots[((a * nk + b) * nk + c) * nk + d] = _orc_bonded(dp)
        coul = OrcCoulomb()
        if spec.coulomb is not None:
            c = spec.coulomb
            r = c.restriction
            rr, s14 = (r[0], r[1]) if isinstance(r, tuple) else (r, 1.0)
            if hasattr(c, "kmax"):
                coul = OrcCoulomb(1, rr, c.kmax, 0, c.cutoff, c.alpha, s14)
            else:
                coul = OrcCoulomb(2, rr, 0, 0, c.cutoff, 0.0, s14)
        desc = OrcDesc()
        desc.n = self.n
        desc.positions = _ptr(pos)
        desc.kinds = _ptr(kinds)
        desc.charges = _ptr(charges)
        desc.masses = _ptr(masses)
        desc.molecules = _ptr(mols)
        desc.n_bonds = len(bonds) // 2
        desc.bonds = _ptr(bonds) if len(bonds) else None
        desc.n_kinds = nk
        desc.pairs = pairs
        desc.bond_pots = bpots
        desc.angle_pots = apots
        desc.dihedral_pots = dpots
        desc.coulomb = coul
        desc.cell = (ctypes.c_double * 3)(*spec.cell.lengths)
        tric = getattr(spec.cell, "shape", "orthorhombic") == "triclinic"
        desc.cell_shape = CELL_TRICLINIC if tric else CELL_ORTHORHOMBIC
        if tric:
            desc.cell_matrix = (ctypes.c_double * 9)(*[float(x) for x in spec.cell.matrix().ravel()])
        self.h = lib.orc_create(ctypes.byref(desc))
        self.masses = masses

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_destroy(self.h)
        except Exception:
            pass

    def set_positions(self, pos) -> None:
        pos = _state_array(pos, self.n)
        self.lib.orc_set_positions(self.h, _ptr(pos))

    def energy(self, terms: int = TERM_ALL) -> float:
        return self.lib.orc_energy(self.h, terms)

    def forces(self, terms: int = TERM_ALL) -> np.ndarray:
        f = np.zeros((self.n, 3))
        self.lib.orc_forces(self.h, terms, _ptr(f))
        return f

    def virial(self, terms: int = TERM_ALL) -> np.ndarray:
        v = np.zeros(9)
        self.lib.orc_virial(self.h, terms, _ptr(v))
        return v.reshape(3, 3)

    def molecular_virial(self, terms: int = TERM_ALL) -> np.ndarray:
        """MolecularVirial (sys/compute.rs:278-362)."""
        v = np.zeros(9)
        self.lib.orc_molecular_virial(self.h, terms, _ptr(v))
        return v.reshape(3, 3)

    def pairset(self, family: int) -> np.ndarray:
        count = self.lib.orc_pairset(self.h, family, None, 0)
        out = np.zeros(2 * max(count, 1), dtype=np.int32)
        self.lib.orc_pairset(self.h, family, _ptr(out), count)
        return out[: 2 * count].reshape(-1, 2)

    def dihedrals(self) -> np.ndarray:
        n = self.lib.orc_n_dihedrals(self.h)
        out = np.zeros(4 * max(n, 1), dtype=np.int32)
        self.lib.orc_dihedrals(self.h, _ptr(out))
        return out[: 4 * n].reshape(-1, 4)

    def angles(self) -> np.ndarray:
        n = self.lib.orc_n_angles(self.h)
        out = np.zeros(3 * max(n, 1), dtype=np.int32)
        self.lib.orc_angles(self.h, _ptr(out))
        return out[: 3 * n].reshape(-1, 3)

    def velocity_verlet(self, pos, vel, acc, dt, nsteps, temperature=0.0, tau=0.0):
        pos = _state_array(pos, self.n, copy=True)
        vel = _state_array(vel, self.n, copy=True)
        acc = _state_array(acc, self.n, copy=True)
        self.lib.orc_velocity_verlet(self.h, _ptr(pos), _ptr(vel), _ptr(acc), dt, nsteps, temperature, tau)
        return pos, vel, acc

    def md_run(self, pos, vel, state, nsteps, integrator=0, dt=1.0, thermostat=0, temperature=0.0, tau=0.0,
               tolerance=0.0, seed=0, count=0, controls=0):
        """MolecularDynamics::propagate for `nsteps` steps (see orc_md_run);
        returns (positions, velocities, state, count)."""
        pos = _state_array(pos, self.n, copy=True)
        vel = _state_array(vel, self.n, copy=True)
        state = _state_array(state, self.n, copy=True)
        c = ctypes.c_uint64(count)
        self.lib.orc_md_run(self.h, _ptr(pos), _ptr(vel), _ptr(state), integrator, dt, thermostat, temperature,
                            tau, tolerance, seed & (2 ** 64 - 1), ctypes.byref(c), controls, nsteps)
        return pos, vel, state, c.value

    def verlet_setup(self, pos, vel, dt) -> np.ndarray:
        pos = _state_array(pos, self.n)
        vel = _state_array(vel, self.n)
        prev = np.zeros_like(pos)
        self.lib.orc_verlet_setup(self.h, _ptr(pos), _ptr(vel), dt, _ptr(prev))
        return prev

    def kinetic_energy(self, vel) -> float:
        vel = _state_array(vel, self.n)
        return self.lib.orc_kinetic_energy(self.h, _ptr(vel))

    def temperature(self, vel) -> float:
        vel = _state_array(vel, self.n)
        return self.lib.orc_temperature(self.h, _ptr(vel))

    def set_cell(self, lengths) -> None:
        self.lib.orc_set_cell(self.h, *[float(x) for x in lengths])

    def set_cell_matrix(self, matrix, triclinic: bool) -> None:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64).reshape(9))
        self.lib.orc_set_cell_matrix(self.h, _ptr(m), CELL_TRICLINIC if triclinic else CELL_ORTHORHOMBIC)

    def cell(self) -> np.ndarray:
        """The orthorhombic lengths (the diagonal of the cell matrix)."""
        out = np.zeros(3)
        self.lib.orc_get_cell(self.h, _ptr(out))
        return out

    def cell_matrix(self) -> np.ndarray:
        out = np.zeros(9)
        self.lib.orc_get_cell_matrix(self.h, _ptr(out))
        return out.reshape(3, 3)

    def cell_apply(self, v, mode: str) -> np.ndarray:
        """UnitCell::vector_image ("image"), wrap_vector ("wrap") or
        cartesian(fractional(v)) ("roundtrip") of one vector."""
        x = np.ascontiguousarray(np.asarray(v, dtype=np.float64).copy())
        self.lib.orc_cell_apply(self.h, _ptr(x), {"image": 0, "wrap": 1, "roundtrip": 2}[mode])
        return x

    def cell_info(self):
        """(UnitCell::lengths, UnitCell::volume) of the oracle's cell."""
        lengths, volume = np.zeros(3), np.zeros(1)
        self.lib.orc_cell_info(self.h, _ptr(lengths), _ptr(volume))
        return lengths, float(volume[0])

    def berendsen_barostat(self, pos, vel, acc, eta, dt, pressure, tau, nsteps, temperature=0.0,
                           tau_thermostat=0.0):
        """BerendsenBarostat::integrate (+ an optional Berendsen thermostat) for
        `nsteps` steps; returns (positions, velocities, accelerations, eta, cell
        lengths).  Raises where the reference panics."""
        pos = _state_array(pos, self.n, copy=True)
        vel = _state_array(vel, self.n, copy=True)
        acc = _state_array(acc, self.n, copy=True)
        e = ctypes.c_double(eta)
        rc = self.lib.orc_berendsen_barostat_run(self.h, _ptr(pos), _ptr(vel), _ptr(acc), ctypes.byref(e), dt,
                                                 pressure, tau, temperature, tau_thermostat, nsteps)
        if rc:
            raise RuntimeError("Tried to decrease the cell size in Berendesen barostat but the new size is "
                               "smaller than the interactions cut off radius.")
        return pos, vel, acc, e.value, self.cell()

    def aniso_barostat(self, pos, vel, acc, eta, dt, stress, tau, nsteps):
        """AnisoBerendsenBarostat::integrate for `nsteps` steps; returns
        (positions, velocities, accelerations, eta (3 x 3), cell matrix).
        Raises where the reference panics."""
        pos = _state_array(pos, self.n, copy=True)
        vel = _state_array(vel, self.n, copy=True)
        acc = _state_array(acc, self.n, copy=True)
        e = np.ascontiguousarray(np.asarray(eta, dtype=np.float64).reshape(9).copy())
        st = np.ascontiguousarray(np.asarray(stress, dtype=np.float64).reshape(9))
        rc = self.lib.orc_aniso_barostat_run(self.h, _ptr(pos), _ptr(vel), _ptr(acc), _ptr(e), dt, _ptr(st), tau,
                                             nsteps)
        if rc:
            raise RuntimeError("Tried to decrease the cell size in anisotropic Berendesen barostat but the new "
                               "size is smaller than the interactions cut off radius.")
        return pos, vel, acc, e.reshape(3, 3), self.cell_matrix()

    def cache_init(self) -> None:
        self.lib.orc_cache_init(self.h)

    def cache_energy(self) -> float:
        return self.lib.orc_cache_energy(self.h)

    def move_molecule_cost(self, molid: int, newpos) -> float:
        newpos = np.ascontiguousarray(newpos, dtype=np.float64)
        return self.lib.orc_move_molecule_cost(self.h, molid, _ptr(newpos))

    def cache_update(self) -> None:
        self.lib.orc_cache_update(self.h)

    def move_all_molecules_cost(self, cell, newpos) -> float:
        """`cell`: the new cell's 3 x 3 matrix, or its three orthorhombic lengths."""
        cell = np.asarray(cell, dtype=np.float64)
        if cell.size == 3:
            cell = np.diag(cell)
        cell = np.ascontiguousarray(cell.reshape(9))
        newpos = _state_array(newpos, self.n)
        return self.lib.orc_move_all_molecules_cost(self.h, _ptr(cell), _ptr(newpos))

    def cache_restore(self) -> None:
        self.lib.orc_cache_restore(self.h)


def _orc_bonded(pot) -> OrcBonded:
    kind, par = pot._params()
    if kind == MORSE:  # Morse {a, x0, depth}
        return OrcBonded(kind, 0, par[2], par[1], par[0])
    k, x0, extra = par
    return OrcBonded(kind, int(extra) if kind == TORSION else 0, k, x0, 0.0)


NULL, HARMONIC, MORSE, COSINE_HARMONIC, TORSION = 1, 4, 6, 10, 11


def bonded_eval(kind: int, k: float, x0: float, x: float, n: int = 0, a: float = 0.0):
    """(energy, force) of a bond / angle / dihedral potential at x (Morse:
    k = depth, width a)."""
    e, f = ctypes.c_double(), ctypes.c_double()
    p = OrcBonded(kind, n, k, x0, a)
    load().orc_bonded_eval(ctypes.byref(p), x, ctypes.byref(e), ctypes.byref(f))
    return e.value, f.value


def dihedral_geometry(r1, r2, r3, r4, cell=(1e9, 1e9, 1e9)):
    """UnitCell::dihedral_and_derivatives: (phi, [d1, d2, d3, d4])."""
    arr = [np.ascontiguousarray(r, dtype=np.float64) for r in (r1, r2, r3, r4)]
    c = np.ascontiguousarray(cell, dtype=np.float64)
    phi = ctypes.c_double()
    d = np.zeros(12)
    load().orc_dihedral_geometry(_ptr(c), *[_ptr(a) for a in arr], ctypes.byref(phi), _ptr(d))
    return phi.value, d.reshape(4, 3)


def pair_eval(potential_type: int, params, cutoff: float, r: float, shifted: bool = False,
              tail: bool = False, table=None):
    """(energy, force, tail_energy, tail_virial) of one PairInteraction at r;
    table = (size, max) evaluates TableComputation::new(potential, size, max)."""
    p0, p1, p2, p3, p4 = (list(params) + [0.0] * 5)[:5]
    tsize, tmax = table if table else (0, 0.0)
    pair = OrcPair(potential_type, int(shifted), 0, int(tail), p0, p1, p2, cutoff, 1.0, p3, p4, tsize, 0, tmax)
    out = [ctypes.c_double() for _ in range(4)]
    load().orc_pair_eval(ctypes.byref(pair), r, *[ctypes.byref(o) for o in out])
    return tuple(o.value for o in out)


def set_threads(n: int) -> None:
    load().orc_set_threads(n)


def num_threads() -> int:
    return load().orc_num_threads()
