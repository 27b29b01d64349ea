"""The oracle's integrators, thermostats and controls against the reference's
own tests (lumol-sim/src/md/controls.rs tests, lumol-sim/tests/thermostats.rs,
tests/md-helium.rs energy bounds).  CPU only."""
import numpy as np

import lumol_gb300 as lg
import oracle
from lumol_gb300 import workloads
from lumol_gb300.units import K_BOLTZMANN

VV, VERLET, LEAP = 0, 1, 2
NONE, BERENDSEN, RESCALE, CSVR = 0, 1, 2, 3
REMOVE_TRANSLATION, REWRAP, REMOVE_ROTATION = 1, 2, 4


def two_silver(x1):
    s = lg.System(lg.UnitCell.cubic(10.0))
    s.add_particles(["Ag", "Ag"], np.array([[0.0, 0.0, 0.0], x1]), masses=[107.8682, 107.8682])
    return s


def test_remove_translation_literals(oracle_lib):
    # controls.rs:95-107
    s = two_silver([1.0, 1.0, 1.0])
    v = np.array([[1.0, 2.0, 0.0], [1.0, 0.0, 0.0]])
    orc = oracle.Oracle(s)
    _, v1, _, _ = orc.md_run(s.positions, v, np.zeros((2, 3)), 1, dt=1e-3, controls=REMOVE_TRANSLATION)
    assert v1.tolist() == [[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]]


def test_remove_rotation_literals(oracle_lib):
    # controls.rs:109-122 (dt = 0: the step leaves the positions as they are)
    s = two_silver([1.0, 0.0, 0.0])
    v = np.array([[0.0, 1.0, 0.0], [0.0, -1.0, 2.0]])
    orc = oracle.Oracle(s)
    _, v1, _, _ = orc.md_run(s.positions, v, np.zeros((2, 3)), 1, dt=0.0, controls=REMOVE_ROTATION)
    assert v1.tolist() == [[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]]


def test_rewrap_literals(oracle_lib):
    # controls.rs:125-131
    s = two_silver([15.0, 0.0, 0.0])
    orc = oracle.Oracle(s)
    x1, _, _, _ = orc.md_run(s.positions, np.zeros((2, 3)), np.zeros((2, 3)), 1, dt=1.0, controls=REWRAP)
    assert x1.tolist() == [[0.0, 0.0, 0.0], [5.0, 0.0, 0.0]]


def helium_gas(n_side=10, temperature=300.0, seed=42):
    """The ideal gas of lumol-sim/tests/thermostats.rs:14-31: helium on a
    2 A grid in a 20 A cubic cell, velocities at exactly `temperature`."""
    s = lg.System(lg.UnitCell.cubic(2.0 * n_side))
    grid = np.array([[i, j, k] for i in range(n_side) for j in range(n_side) for k in range(n_side)], float) * 2.0
    s.add_particles(["He"] * len(grid), grid)
    orc = oracle.Oracle(s)
    v = np.random.default_rng(seed).normal(size=grid.shape)
    v -= v.mean(axis=0)
    v *= np.sqrt(temperature / orc.temperature(v))
    return s, orc, v


def test_rescale_thermostat_literals(oracle_lib):
    # lumol-sim/tests/thermostats.rs:34-49: no rescaling within the tolerance, exact T outside it
    s, orc, v = helium_gas()
    assert abs(orc.temperature(v) - 300.0) < 1e-12
    x = s.positions
    _, v1, _, _ = orc.md_run(x, v, np.zeros_like(x), 1, dt=1.0, thermostat=RESCALE, temperature=250.0,
                             tolerance=100.0)
    assert abs(orc.temperature(v1) - 300.0) < 1e-12
    _, v2, _, _ = orc.md_run(x, v, np.zeros_like(x), 1, dt=1.0, thermostat=RESCALE, temperature=250.0,
                             tolerance=10.0)
    assert abs(orc.temperature(v2) - 250.0) < 1e-12


def test_csvr_mean_kinetic_energy(oracle_lib):
    """lumol-sim/tests/thermostats.rs:80-117 checks <K> = dof kT / 2 with the
    reference's own noise sequence; with this noise stream the same statement
    holds statistically: 64 atoms, tau = 10 steps, 4000 steps after 200 of
    equilibration, within 3 % (five standard errors)."""
    s, orc, v = helium_gas(n_side=4, temperature=300.0)
    x = s.positions
    state = np.zeros_like(x)
    x, v, state, count = orc.md_run(x, v, state, 200, dt=1.0, thermostat=CSVR, temperature=250.0, tau=10.0,
                                    seed=7)
    assert count == 200
    kinetic = []
    for _ in range(400):
        x, v, state, count = orc.md_run(x, v, state, 10, dt=1.0, thermostat=CSVR, temperature=250.0,
                                        tau=10.0, seed=7, count=count)
        kinetic.append(orc.kinetic_energy(v))
    dof = 3 * s.size
    expected = dof * K_BOLTZMANN * 250.0 / 2.0
    assert abs(np.mean(kinetic) / expected - 1.0) < 0.03


def total_energy(orc, x, v):
    orc.set_positions(x)
    return orc.energy() + orc.kinetic_energy(v)


def test_integrators_conserve_energy(oracle_lib):
    """tests/md-helium.rs:18-64 bounds the NVE drift of VelocityVerlet and
    LeapFrog by 5e-3 and of Verlet by 1e-2 (relative); here on an argon-like
    LJ fluid, 300 steps of 1 fs."""
    s = workloads.lj_replica(256, 0.8, 120.0, 3)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    e0 = total_energy(orc, x0, v0)
    for integrator, bound in ((VV, 5e-3), (LEAP, 5e-3), (VERLET, 1e-2)):
        state = orc.verlet_setup(x0, v0, 1.0) if integrator == VERLET else np.zeros_like(x0)
        x, v, _, _ = orc.md_run(x0, v0, state, 300, integrator=integrator, dt=1.0)
        assert abs((total_energy(orc, x, v) - e0) / e0) < bound, integrator


def test_berendsen_barostat_sequence(oracle_lib):
    """The oracle's BerendsenBarostat follows integrators.rs:213-250 step by step:
    v += dt/2 a; x *= eta; x += v dt; the cell matrix times eta^3; the pressure
    (N_f k_B T + Tr W) / (3 V) at the new positions with the half-step
    velocities (compute.rs:399-431) sets eta^3 = 1 - 7372 / tau (P0 - P) for
    the next step; then the forces and the second half kick.  Restated here
    with the oracle's own virial, forces and temperature."""
    s = workloads.argon_fcc()
    s.positions = s.positions + np.random.default_rng(3).uniform(-0.2, 0.2, size=(s.size, 3))
    dt, P0, tau = 1.0, 4e-5, 20.0
    orc = oracle.Oracle(s)
    got = orc.berendsen_barostat(s.positions, s.velocities, np.zeros((s.size, 3)), 1.0, dt, P0, tau, 2)

    ref = oracle.Oracle(s)
    x, v, a, eta = s.positions.copy(), s.velocities.copy(), np.zeros((s.size, 3)), 1.0
    L = np.array(s.cell.lengths)
    m = s.masses[:, None]
    for _ in range(2):
        v = v + 0.5 * dt * a
        x = x * eta
        x = x + v * dt
        L = L * (eta * eta * eta)
        ref.set_cell(L)
        ref.set_positions(x)
        w = ref.virial()
        dof = 3 * s.size
        T = 2.0 * (0.5 * np.sum(m * v * v)) / (dof * K_BOLTZMANN)
        P = (dof * K_BOLTZMANN * T + np.trace(w)) / (3.0 * np.prod(L))
        eta = np.cbrt(1.0 - 7372.0 / tau * (P0 - P))
        a = ref.forces() / m
        v = v + 0.5 * dt * a
    xg, vg, ag, etag, cellg = got
    assert abs(etag - eta) < 1e-14 and np.allclose(cellg, L, rtol=1e-15, atol=0)
    assert np.abs(xg - x).max() < 1e-12 and np.abs(vg - v).max() < 1e-14
    assert etag != 1.0 and not np.allclose(L, s.cell.lengths)
