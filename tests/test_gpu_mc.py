"""Monte Carlo move costs on the GPU against the oracle's EnergyCache
(sys/cache.rs:145-220) with Ewald / Wolf GlobalCache costs."""
import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("coulomb", ["none", "ewald", "wolf"])
def test_move_costs_match_oracle(coulomb):
    s = systems.chains(27, 24.0, 3, lg.PairRestriction.INTER_MOLECULAR,
                       coulomb={"none": None, "ewald": lg.Ewald(9.0, 5, 0.35), "wolf": lg.Wolf(9.0)}[coulomb])
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = s.mc_init()
    assert abs(e0 - orc.cache_energy()) <= 1e-10 * abs(e0)
    rng = np.random.default_rng(5)
    # distinct molecules: the reference keeps its e^{ik.r} table stale for a molecule
    # that moved before (ewald.rs:826-830), the engine refreshes it
    for molid in (3, 11, 20, 7):
        lo, hi = s.molecule_range(molid)
        newpos = s.positions[lo:hi] + rng.uniform(-0.5, 0.5, size=3)
        cost = s.move_molecule_cost(molid, newpos)
        cost_ref = orc.move_molecule_cost(molid, newpos)
        assert abs(cost - cost_ref) <= 1e-10 * abs(e0), (cost, cost_ref)
        wrapped = s.wrap_molecule(molid, newpos)
        e_gpu = s.mc_update(molid, wrapped)
        pos = s.positions.copy()
        orc.set_positions(pos)
        orc.cache_update()
        assert abs(e_gpu - orc.cache_energy()) <= 1e-9 * abs(e0)


def test_cached_energy_equals_fresh_energy_after_many_moves():
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    mc = lg.MonteCarlo(300.0, lg.Translate(0.3), seed=1)
    mc.setup(s)
    for _ in range(300):
        mc.propagate(s)
    fresh = s.potential_energy()
    assert mc.accepted > 0
    assert abs(mc.energy - fresh) <= 1e-9 * abs(fresh)


def test_rotate_and_translate_moves_on_water():
    """Rotate (mc/moves/rotate.rs) with Translate on rigid water with Ewald:
    rotations keep every molecule's geometry, some of each kind are accepted,
    and the cached energy equals a fresh evaluation after 300 moves."""
    s = workloads.water_box(n_side=4, length=14.0, seed=2, cutoff=6.5, alpha=0.45, kmax=6)
    s.set_bond_potential(("H", "O"), lg.NullPotential())
    s.set_angle_potential(("H", "O", "H"), lg.NullPotential())
    mc = lg.MonteCarlo(300.0, [(lg.Translate(0.3), 1.0), (lg.Rotate(0.6), 1.0)], seed=4)
    mc.setup(s)
    assert s.simulated_degrees_of_freedom == "molecules" and s.temperature() == 300.0

    def geometry(x):
        x = x.reshape(-1, 3, 3)
        return np.stack([np.linalg.norm(x[:, 1] - x[:, 0], axis=1), np.linalg.norm(x[:, 2] - x[:, 0], axis=1),
                         np.linalg.norm(x[:, 2] - x[:, 1], axis=1)])

    g0 = geometry(s.positions)
    for _ in range(300):
        mc.propagate(s)
    assert mc.accepted > 0 and mc.accepted < mc.attempted
    assert np.abs(geometry(s.positions) - g0).max() < 1e-12
    fresh = s.potential_energy()
    assert abs(mc.energy - fresh) <= 1e-9 * abs(fresh)


def test_update_without_cost_is_an_error():
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    s.mc_init()
    with pytest.raises(lg.EngineError, match="without call a"):
        s.mc_update(0, s.positions[0:1])


def test_accepted_rotation_is_not_wrapped():
    """Rotate::apply copies the rotated positions as they are (rotate.rs:91-96),
    unlike Translate::apply, which wraps the centre of mass into the cell: a
    molecule whose centre of mass lies outside the cell stays outside after an
    accepted rotation, at com + R (x - com)."""
    s = workloads.water_box(n_side=3, length=14.0, seed=3, cutoff=6.5, alpha=0.45, kmax=5)
    s.set_bond_potential(("H", "O"), lg.NullPotential())
    s.set_angle_potential(("H", "O", "H"), lg.NullPotential())
    pos = s.positions.copy()
    lo, hi = s.molecule_range(4)
    pos[lo:hi] += np.array([14.0, -14.0, 0.0])  # the same periodic image, centre of mass outside
    s.positions = pos
    # a huge temperature accepts every move
    mc = lg.MonteCarlo(1e12, lg.Rotate(0.5), seed=7)
    mc.setup(s)
    rotated_outside = 0
    for _ in range(400):
        before = s.positions.copy()
        mc.propagate(s)
        after = s.positions
        moved = np.flatnonzero(np.any(after != before, axis=1))
        if moved.size == 0:
            continue
        mol = int(s.molecules[moved[0]])
        rotated_outside += mol == 4
        if rotated_outside >= 3:
            break
        a, b = s.molecule_range(mol)
        m = s.masses[a:b, None]
        com_before = (m * before[a:b]).sum(axis=0) / m.sum()
        com_after = (m * after[a:b]).sum(axis=0) / m.sum()
        assert np.abs(com_after - com_before).max() < 1e-9, (mol, com_before, com_after)
    lo, hi = s.molecule_range(4)
    m = s.masses[lo:hi, None]
    com = (m * s.positions[lo:hi]).sum(axis=0) / m.sum()
    assert rotated_outside >= 3
    assert com[0] > 14.0 and com[1] < 0.0
    assert mc.accepted == mc.attempted
    fresh = s.potential_energy()
    assert abs(mc.energy - fresh) <= 1e-9 * abs(fresh)
