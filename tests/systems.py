"""Small systems of the reference's unit tests, rebuilt with the engine's
System description (no GPU is touched until a computation is asked for)."""
from __future__ import annotations

import numpy as np

import lumol_gb300 as lg
from lumol_gb300 import units

import refdata


def nacl_pair() -> lg.System:
    """energy/global/ewald.rs:963-972 and wolf.rs tests: Cl at 0, Na at 1.5 A, cell 20."""
    s = lg.System(lg.UnitCell.cubic(20.0))
    s.add_particle("Cl", [0.0, 0.0, 0.0], charge=-1.0)
    s.add_particle("Na", [1.5, 0.0, 0.0], charge=1.0)
    return s


def ewald_water() -> lg.System:
    """energy/global/ewald.rs:975-995: one water molecule in a 20 A cell."""
    s = lg.System(lg.UnitCell.cubic(20.0))
    s.add_molecule(["O", "H", "H"], [[0.0, 0.0, 0.0], [-0.7, -0.7, 0.3], [0.3, -0.3, -0.8]],
                   bonds=[(0, 1), (0, 2)], charges=[-0.8476, 0.4238, 0.4238])
    return s


def evaluator_system() -> lg.System:
    """sys/energy.rs:171-222: four bonded F atoms with LJ + tail, harmonic bond and angle."""
    s = lg.System(lg.UnitCell.cubic(10.0))
    s.add_molecule(["F"] * 4, [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [1.0, 1.0, 0.0], [2.0, 1.0, 0.0]],
                   bonds=[(0, 1), (1, 2), (2, 3)])
    pair = lg.PairInteraction(
        lg.LennardJones(epsilon=units.from_(100.0, "kJ/mol/A^2"), sigma=units.from_(0.8, "A")), 5.0)
    pair.enable_tail_corrections()
    s.set_pair_potential(("F", "F"), pair)
    s.set_bond_potential(("F", "F"), lg.Harmonic(k=units.from_(100.0, "kJ/mol/A^2"), x0=units.from_(2.0, "A")))
    s.set_angle_potential(("F", "F", "F"),
                          lg.Harmonic(k=units.from_(100.0, "kJ/mol/deg^2"), x0=units.from_(88.0, "deg")))
    s.set_pair_potential(("H", "O"), lg.PairInteraction(lg.NullPotential(), 0.0))
    return s


def nist_lj(xyz: str, cutoff: float, tail: bool) -> lg.System:
    """tests/nist-lj.rs:14-58 with the configuration of tests/data/nist-lj."""
    names, pos, cell = refdata.read_xyz(xyz)
    s = lg.System(lg.UnitCell.ortho(*cell))
    s.add_particles(names, pos, masses=[1.0] * len(names))
    lj = lg.PairInteraction(lg.LennardJones(epsilon=1.0, sigma=1.0), cutoff)
    if tail:
        lj.enable_tail_corrections()
    s.set_pair_potential(("H", "H"), lj)
    return s


def nist_spce(xyz: str, cutoff: float, lammps: tuple | None = None) -> lg.System:
    """tests/nist-spce.rs:24-100: SPC/E water, NIST or LAMMPS parameters."""
    names, pos, cell = refdata.read_xyz(xyz)
    s = lg.System(lg.UnitCell.ortho(*cell))
    for m in range(len(names) // 3):
        s.add_molecule(names[3 * m: 3 * m + 3], pos[3 * m: 3 * m + 3], bonds=[(0, 1), (0, 2)],
                       charges=[-2.0 * 0.42380 if nm == "O" else 0.42380 for nm in names[3 * m: 3 * m + 3]])
    lj = lg.PairInteraction(lg.LennardJones(epsilon=78.19743111 * units.K_BOLTZMANN, sigma=3.16555789), cutoff)
    if lammps is None:
        lj.enable_tail_corrections()
    s.set_pair_potential(("O", "O"), lj)
    s.set_pair_potential(("O", "H"), lg.PairInteraction(lg.NullPotential(), cutoff))
    s.set_pair_potential(("H", "H"), lg.PairInteraction(lg.NullPotential(), cutoff))
    if lammps is None:
        alpha = 5.6 / min(cell)
        ewald = lg.Ewald(cutoff, 5, alpha)
    else:
        kmax, alpha = lammps
        ewald = lg.Ewald(cutoff, kmax, alpha)
    ewald.set_restriction(lg.PairRestriction.INTER_MOLECULAR)
    s.set_coulomb_potential(ewald)
    return s


def _family_interactions(family: str, cutoff: float):
    """Three PairInteractions of one potential family for the kinds (Ar, Ar),
    (Ar, Kr), (Kr, Kr): plain, shifted, and with tail corrections."""
    eps = units.from_(0.996, "kJ/mol")
    pots = {
        "lj": (lg.LennardJones(3.405, eps), lg.LennardJones(3.6, 1.3 * eps), lg.LennardJones(3.8, 1.6 * eps)),
        "buckingham": (lg.Buckingham(5000.0, 40.0, 0.3), lg.Buckingham(6000.0, 50.0, 0.32),
                       lg.Buckingham(7000.0, 60.0, 0.35)),
        "bmh": (lg.BornMayerHuggins(0.2, 40.0, 60.0, 3.0, 0.3), lg.BornMayerHuggins(0.25, 50.0, 70.0, 3.1, 0.32),
                lg.BornMayerHuggins(0.3, 60.0, 80.0, 3.2, 0.35)),
        "morse": (lg.Morse(1.5, 3.8, eps), lg.Morse(1.4, 4.0, 1.3 * eps), lg.Morse(1.3, 4.2, 1.6 * eps)),
        "gaussian": (lg.Gaussian(2.0 * eps, 0.08), lg.Gaussian(2.5 * eps, 0.07), lg.Gaussian(3.0 * eps, 0.06)),
        "mie": (lg.Mie(3.405, eps, 12.0, 6.0), lg.Mie(3.6, 1.3 * eps, 12.5, 6.5), lg.Mie(3.8, 1.6 * eps, 14.0, 7.0)),
        # TableComputation of LJ / Mie / LJ, 4000 points up to 10 A
        "table": (lg.TableComputation(lg.LennardJones(3.405, eps), 4000, 10.0),
                  lg.TableComputation(lg.Mie(3.6, 1.3 * eps, 12.5, 6.5), 4000, 10.0),
                  lg.TableComputation(lg.LennardJones(3.8, 1.6 * eps), 4000, 10.0)),
    }[family]
    if family == "lj":  # the historical LJ fluid: shifted, tail, plain
        tail = lg.PairInteraction(pots[1], cutoff)
        tail.enable_tail_corrections()
        return lg.PairInteraction.shifted(pots[0], cutoff), tail, lg.PairInteraction(pots[2], cutoff)
    tail = lg.PairInteraction(pots[2], cutoff)
    tail.enable_tail_corrections()
    return lg.PairInteraction(pots[0], cutoff), lg.PairInteraction.shifted(pots[1], cutoff), tail


def random_lj_fluid(n: int, density: float, seed: int, cutoff: float, family: str = "lj",
                    precision: str = "fp64") -> lg.System:
    """Jittered simple-cubic fluid of `n` particles (two kinds) at `density` (1/A^3),
    with pair potentials of one family ("lj", "buckingham", "bmh", "morse",
    "gaussian", "mie", "table")."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    length = (n / density) ** (1.0 / 3.0)
    grid = np.array([[i, j, k] for i in range(side) for j in range(side) for k in range(side)][:n], dtype=float)
    pos = (grid + 0.5 + rng.uniform(-0.2, 0.2, size=grid.shape)) * (length / side)
    # unwrapped positions: shift some atoms by whole cell vectors
    pos += rng.integers(-2, 3, size=pos.shape) * length
    names = ["Ar" if i % 3 else "Kr" for i in range(n)]
    s = lg.System(lg.UnitCell.cubic(length), precision=precision)
    s.add_particles(names, pos)
    aa, ak, kk = _family_interactions(family, cutoff)
    s.set_pair_potential(("Ar", "Ar"), aa)
    s.set_pair_potential(("Ar", "Kr"), ak)
    s.set_pair_potential(("Kr", "Kr"), kk)
    return s


def chains(n_mol: int, length: float, seed: int, restriction, coulomb=None, dihedrals: bool = False) -> lg.System:
    """Flexible 5-atom chains with charges, for bond-path restrictions; with
    `dihedrals`, a Torsion on C-C-O-C, a CosineHarmonic on C-O-C-N and a
    CosineHarmonic O-C-N angle."""
    rng = np.random.default_rng(seed)
    s = lg.System(lg.UnitCell.cubic(length))
    side = int(np.ceil(n_mol ** (1.0 / 3.0)))
    m = 0
    for i in range(side):
        for j in range(side):
            for k in range(side):
                if m == n_mol:
                    break
                base = (np.array([i, j, k]) + 0.5) * length / side
                pos = base + np.array([[0.0, 0, 0], [1.2, 0.2, 0], [2.1, 1.1, 0.1], [3.2, 1.0, 0.9], [4.1, 1.8, 1.2]])
                pos = pos - pos.mean(axis=0) + base + rng.uniform(-0.1, 0.1, size=(5, 3))
                s.add_molecule(["C", "C", "O", "C", "N"], pos, bonds=[(0, 1), (1, 2), (2, 3), (3, 4)],
                               charges=[0.3, -0.2, -0.4, 0.1, 0.2])
                m += 1
    eps = units.from_(0.5, "kJ/mol")
    for a, b, sig in [("C", "C", 3.4), ("C", "O", 3.2), ("C", "N", 3.3), ("O", "O", 3.0), ("O", "N", 3.1),
                      ("N", "N", 3.25)]:
        p = lg.PairInteraction(lg.LennardJones(sig, eps), 7.0)
        p.set_restriction(restriction)
        s.set_pair_potential((a, b), p)
    s.set_bond_potential(("C", "C"), lg.Harmonic(k=units.from_(2000.0, "kJ/mol/A^2"), x0=1.2))
    s.set_bond_potential(("C", "O"), lg.Harmonic(k=units.from_(2500.0, "kJ/mol/A^2"), x0=1.3))
    s.set_bond_potential(("C", "N"), lg.Harmonic(k=units.from_(2200.0, "kJ/mol/A^2"), x0=1.25))
    s.set_angle_potential(("C", "C", "O"), lg.Harmonic(k=units.from_(300.0, "kJ/mol/rad^2"), x0=1.9))
    s.set_angle_potential(("C", "O", "C"), lg.Harmonic(k=units.from_(320.0, "kJ/mol/rad^2"), x0=1.95))
    s.set_angle_potential(("O", "C", "N"), lg.Harmonic(k=units.from_(280.0, "kJ/mol/rad^2"), x0=2.0))
    if dihedrals:
        s.set_angle_potential(("O", "C", "N"), lg.CosineHarmonic(k=units.from_(250.0, "kJ/mol"), x0=2.0))
        s.set_dihedral_potential(("C", "C", "O", "C"), lg.Torsion(k=units.from_(5.0, "kJ/mol"), delta=0.4, n=3))
        s.set_dihedral_potential(("N", "C", "O", "C"), lg.CosineHarmonic(k=units.from_(40.0, "kJ/mol"), x0=1.2))
    if coulomb is not None:
        coulomb.set_restriction(restriction)
        s.set_coulomb_potential(coulomb)
    return s
