"""MolecularVirial (lumol-core/src/sys/compute.rs:278-362) on the GPU and in
the oracle.

The reference has no known-answer test for it (its benches time it,
benches/{water,nacl,argon,propane}.rs), so the oracle's restatement is pinned
by two properties of the definition: for one-atom molecules it equals the
atomic virial term by term, and for rigid molecules its trace is minus the
derivative of the potential energy when the centres of mass and the cell are
scaled together (the virial theorem the molecular definition is built for),
where the image of the centres' separation agrees with the atoms' one.
The GPU is then held to the oracle at 1e-10 relative."""
import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import units, workloads

PAIRS, TAIL, REAL, KSPACE = lg.LG_TERM_PAIRS, lg.LG_TERM_TAIL, lg.LG_TERM_COUL_REAL, lg.LG_TERM_COUL_KSPACE
TERMS = [PAIRS | TAIL | REAL | KSPACE, PAIRS, TAIL, REAL, KSPACE]


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def small_water(coulomb="ewald", scale=1.0, seed=5):
    """64 water molecules in an 18 A cell, cutoff 6.5 A: every pair of atoms
    within the cutoff belongs to molecules whose centres are closer than half
    the cell, so the image of the centres' separation is the one of the atoms'."""
    s = workloads.water_box(n_side=4, length=18.0, seed=seed, cutoff=6.5, alpha=0.45, kmax=6)
    if coulomb == "wolf":
        w = lg.Wolf(6.5)
        w.set_restriction(lg.PairRestriction.INTER_MOLECULAR)
        s.set_coulomb_potential(w)
    if scale != 1.0:
        x = s.positions.reshape(-1, 3, 3)
        m = s.masses.reshape(-1, 3, 1)
        com = (m * x).sum(axis=1, keepdims=True) / m.sum(axis=1, keepdims=True)
        s.cell = lg.UnitCell.cubic(18.0 * scale)
        s.positions = (x + (scale - 1.0) * com).reshape(-1, 3)
    return s


def nacl(coulomb="ewald"):
    return workloads.nacl_crystal(cells=3, a=5.64, jitter=0.1, seed=2, cutoff=8.0, coulomb=coulomb)


def test_oracle_one_atom_molecules_equal_atomic_virial():
    cases = [systems.random_lj_fluid(400, 0.02, 3, 9.0, family="lj"), nacl(), nacl("wolf")]
    for s in cases:
        orc = oracle.Oracle(s)
        for terms in TERMS:
            atomic, molecular = orc.virial(terms), orc.molecular_virial(terms)
            if np.abs(atomic).max() == 0.0:
                assert np.abs(molecular).max() == 0.0
            else:
                assert _rel(molecular, atomic) < 1e-12, terms


def test_oracle_trace_is_the_centre_of_mass_scaling_derivative():
    """tr W_mol = -dU/d lambda for x_a -> x_a + (lambda - 1) com(a), L -> lambda L
    (pairs, Ewald real space, self and k space; rigid molecules)."""
    terms = PAIRS | REAL | lg.LG_TERM_COUL_SELF | KSPACE
    eps = 1e-5
    energy = {}
    for lam in (1.0 - eps, 1.0 + eps):
        energy[lam] = oracle.Oracle(small_water(scale=lam)).energy(terms)
    dudl = (energy[1.0 + eps] - energy[1.0 - eps]) / (2.0 * eps)
    w = oracle.Oracle(small_water()).molecular_virial(PAIRS | REAL | KSPACE)
    assert abs(np.trace(w) + dudl) / abs(dudl) < 1e-7
    # the atomic virial differs for molecules (it holds the intramolecular forces)
    atomic = oracle.Oracle(small_water()).virial(PAIRS | REAL | KSPACE)
    assert _rel(w, atomic) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water_ewald", "water_wolf", "chains_wolf", "argon", "nacl"])
def test_molecular_virial_matches_oracle(name):
    s = {"water_ewald": lambda: small_water(),
         "water_wolf": lambda: small_water("wolf"),
         "chains_wolf": lambda: systems.chains(27, 24.0, 9, lg.PairRestriction.EXCLUDE13, coulomb=lg.Wolf(8.0)),
         "argon": lambda: systems.random_lj_fluid(400, 0.02, 3, 9.0, family="lj"),
         "nacl": nacl}[name]()
    orc = oracle.Oracle(s)
    for terms in TERMS + [lg.LG_TERM_ALL]:
        gpu, ref = s.molecular_virial(terms), orc.molecular_virial(terms)
        if np.abs(ref).max() < 1e-14:
            assert np.abs(gpu).max() < 1e-14, terms
        else:
            assert _rel(gpu, ref) <= 1e-10, (terms, gpu, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water_ewald", "argon", "nacl"])
def test_molecular_virial_of_mixed_engines(name):
    """A mixed engine evaluates the pair and real-space terms in FP64 on its
    cell-sorted list (each pair once), so they match the oracle at 1e-10; the
    k-space correction takes its FP32-accurate k-space forces (1e-5 of the
    largest entry, the mixed path's virial tolerance)."""
    mixed = {"water_ewald": lambda: workloads.water_box(n_side=4, length=18.0, seed=5, cutoff=6.5, alpha=0.45,
                                                        kmax=6, precision="mixed"),
             "argon": lambda: systems.random_lj_fluid(400, 0.02, 3, 9.0, family="lj", precision="mixed"),
             "nacl": lambda: workloads.nacl_crystal(cells=3, a=5.64, jitter=0.1, seed=2, cutoff=8.0,
                                                    precision="mixed")}[name]()
    orc = oracle.Oracle(mixed)
    for terms in TERMS + [lg.LG_TERM_ALL]:
        gpu, ref = mixed.molecular_virial(terms), orc.molecular_virial(terms)
        tol = 1e-5 if terms & KSPACE else 1e-10
        if np.abs(ref).max() < 1e-14:
            assert np.abs(gpu).max() < 1e-12, terms
        else:
            assert _rel(gpu, ref) <= tol, (terms, _rel(gpu, ref))


def pairs_system():
    """sys/compute.rs tests, test_pairs_system: two F atoms 1.3 A apart in a
    10 A cell with velocities, a Harmonic pair (300 kJ/mol/A^2, 1.2 A) with
    tail corrections at 5 A."""
    s = lg.System(lg.UnitCell.cubic(10.0))
    s.add_particles(["F", "F"], [[0.0, 0.0, 0.0], [1.3, 0.0, 0.0]])
    s.velocities = np.array([[-0.007225222699367925, -0.002405756495275919, 0.0026065109398392215],
                             [0.001179633958023287, 0.003525262341736351, -0.0004132774783154952]])
    pair = lg.PairInteraction(lg.Harmonic(k=units.from_(300.0, "kJ/mol/A^2"), x0=1.2), 5.0)
    pair.enable_tail_corrections()
    s.set_pair_potential(("F", "F"), pair)
    return s


@pytest.mark.gpu
def test_pressure_and_stress_literals():
    """sys/compute.rs tests: temperature 300 K, virial -30 kJ/mol/A * 1.3 A in
    xx, PressureAtTemperature(550 K), Pressure with an external temperature,
    and the stress whose trace / 3 is the pressure."""
    from lumol_gb300.units import K_BOLTZMANN
    s = pairs_system()
    assert abs(s.temperature() - 300.0) < 1e-12
    force = units.from_(30.0, "kJ/mol/A")
    expected = np.zeros((3, 3))
    expected[0, 0] = -force * 1.3
    w = s.virial()
    assert np.abs(w - expected).max() <= 1e-14 * abs(expected[0, 0])
    p = s.pressure_at_temperature(550.0)
    assert abs(p - (2.0 * K_BOLTZMANN * 550.0 / 1000.0 + expected[0, 0] / 3000.0)) <= 1e-14 * abs(p)
    assert s.pressure() == s.pressure_at_temperature(s.temperature())
    s.simulated_temperature(550.0)
    assert s.pressure() == p
    stress = s.stress_at_temperature(550.0)
    assert abs(np.trace(stress) / 3.0 - p) <= 1e-14 * abs(p)
    with pytest.raises(ValueError):
        s.pressure_at_temperature(-4.0)
    # molecules as the degrees of freedom: the molecular definition (one-atom molecules: the same)
    s.simulated_degrees_of_freedom = "molecules"
    assert np.abs(s.virial() - w).max() <= 1e-14 * abs(expected[0, 0])
