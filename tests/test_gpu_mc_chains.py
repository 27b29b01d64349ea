"""Batched Monte Carlo chains (lg_mc_setup / lg_mc_run) against the oracle.

The device chain draws its moves from SplitMix64; the test replays the same
draws through the oracle's EnergyCache (sys/cache.rs:145-220) and Metropolis
rule (mc/monte_carlo.rs:309-312), so accepted moves and final positions can be
compared move for move."""
import math

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
from lumol_gb300 import workloads
from lumol_gb300.batch import Batch, SplitMix64
from lumol_gb300.units import K_BOLTZMANN

pytestmark = pytest.mark.gpu


def replay(system, temperature, delta, seed, moves):
    orc = oracle.Oracle(system)
    orc.cache_init()
    rng = SplitMix64(seed)
    beta = 1.0 / (K_BOLTZMANN * temperature)
    half = delta / math.sqrt(3.0)
    pos = system.positions.copy()
    n = system.size
    L = np.array(system.cell.lengths)
    accepted = 0
    for _ in range(moves):
        i = min(int(rng.uniform() * n), n - 1)
        d = np.array([-half + 2.0 * half * rng.uniform() for _ in range(3)])
        u = rng.uniform()
        new = pos[i] + d
        cost = beta * orc.move_molecule_cost(i, new.reshape(1, 3))
        if cost <= 0.0 or u < math.exp(-cost):
            wrapped = new - np.floor(new / L) * L
            pos[i] = wrapped
            orc.set_positions(pos)
            orc.cache_update()
            accepted += 1
    return pos, orc.cache_energy(), accepted


def test_chains_follow_the_oracle_move_for_move():
    systems = [workloads.lj_replica(300, 0.6, 120.0, 11), workloads.lj_replica(500, 0.8, 90.0, 12)]
    batch = Batch(systems)
    batch.md_setup([1.0, 1.0])
    for s in range(2):
        batch.mc_setup(s, [120.0, 90.0][s], 0.3, 100 + s)
    moves = 400
    batch.mc_run(moves)
    for s, T in enumerate([120.0, 90.0]):
        pos_ref, e_ref, acc_ref = replay(systems[s], T, 0.3, 100 + s, moves)
        energy, acc, att = batch.mc_stats(s)
        pos, _ = batch.state(s)
        assert att == moves
        assert acc == acc_ref
        assert np.abs(pos - pos_ref).max() < 1e-9
        assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chain_energy_tracks_fresh_energy(precision):
    systems = [workloads.lj_replica(n, rho, T, 20 + k, precision)
               for k, (n, rho, T) in enumerate([(200, 0.4, 150.0), (800, 0.9, 100.0), (1500, 0.7, 250.0)])]
    batch = Batch(systems, precision=precision)
    batch.md_setup([1.0] * 3)
    for s in range(3):
        batch.mc_setup(s, [150.0, 100.0, 250.0][s], 0.3, 7 + s)
    batch.mc_run(3000)  # forces several list rebuilds
    for s in range(3):
        energy, acc, att = batch.mc_stats(s)
        assert att == 3000 and acc > 0
        fresh = batch.energy(s)
        tol = 1e-9 if precision == "fp64" else 1e-5
        assert abs(energy - fresh) <= tol * abs(fresh), (energy, fresh)


def test_coulomb_systems_are_rejected():
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    batch = Batch([s])
    with pytest.raises(lg.EngineError, match="pair potentials only"):
        batch.mc_setup(0, 300.0, 0.3, 1)


@pytest.mark.parametrize("family", ["bmh", "morse", "gaussian", "mie", "table"])
def test_chains_with_other_pair_potentials(family):
    """FP64 chains follow the oracle move for move; mixed chains keep their
    running energy within 1e-5 of a fresh evaluation."""
    import systems as fluids
    s = fluids.random_lj_fluid(400, 0.02, 9, 9.0, family=family)
    batch = Batch([s])
    batch.md_setup([1.0])
    batch.mc_setup(0, 300.0, 0.3, 55)
    moves = 300
    batch.mc_run(moves)
    pos_ref, e_ref, acc_ref = replay(s, 300.0, 0.3, 55, moves)
    energy, acc, att = batch.mc_stats(0)
    pos, _ = batch.state(0)
    assert att == moves and acc == acc_ref
    assert np.abs(pos - pos_ref).max() < 1e-9
    assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)
    batch.engine.close()

    m = fluids.random_lj_fluid(400, 0.02, 9, 9.0, family=family, precision="mixed")
    batch = Batch([m], precision="mixed")
    batch.md_setup([1.0])
    batch.mc_setup(0, 300.0, 0.3, 56)
    batch.mc_run(2000)
    energy, acc, att = batch.mc_stats(0)
    fresh = batch.energy(0)
    assert att == 2000 and acc > 0
    assert abs(energy - fresh) <= 1e-5 * abs(fresh), (energy, fresh)
