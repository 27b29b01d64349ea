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


# ---- molecular chains: Translate and Rotate of whole molecules (lg_mc_setup_ex) ---------
def replay_molecular(system, temperature, delta, f_t, theta, f_r, seed, moves, refresh=False):
    """The molecular chain's draws (move by cumulative frequency, molecule,
    displacement or Marsaglia axis + angle, Metropolis number) replayed through
    the oracle's EnergyCache, with the moves applied as Translate (then
    Molecule::wrap) and Rotate (rotate_around_axis) apply them.  `refresh`
    rebuilds the oracle's cache after every accepted move: with Ewald, the
    reference keeps a moved molecule's e^{ik.r} stale (ewald.rs:826-830),
    the engine's chains do not."""
    orc = oracle.Oracle(system)
    orc.cache_init()
    rng = SplitMix64(seed)
    beta = 1.0 / (K_BOLTZMANN * temperature)
    half = delta / math.sqrt(3.0)
    cum_t = f_t / (f_t + f_r) if f_r > 0.0 else 1.0
    pos = system.positions.copy()
    masses = system.masses
    L = np.array(system.cell.lengths)
    nmol = int(system.molecules[-1]) + 1
    accepted = 0
    for _ in range(moves):
        rotate = not (rng.uniform() <= cum_t)
        m = min(int(rng.uniform() * nmol), nmol - 1)
        lo, hi = system.molecule_range(m)
        if not rotate:
            d = [-half + 2.0 * half * rng.uniform() for _ in range(3)]
            new = pos[lo:hi] + np.array(d)
        else:
            x1 = x2 = 0.0
            s = 1.0
            tries = 0
            while tries < 64 and not (s < 1.0):
                x1 = -1.0 + 2.0 * rng.uniform()
                x2 = -1.0 + 2.0 * rng.uniform()
                s = x1 * x1 + x2 * x2
                tries += 1
            axis = [0.0, 0.0, 1.0]
            if s < 1.0:
                f = 2.0 * math.sqrt(1.0 - s)
                axis = [x1 * f, x2 * f, 1.0 - 2.0 * s]
            angle = -theta + 2.0 * theta * rng.uniform()
            norm = math.sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2])
            n = [axis[0] / norm, axis[1] / norm, axis[2] / norm]
            sn, cs = math.sin(angle), math.cos(angle)
            omc = 1.0 - cs
            xy, xz, yz = n[0] * n[1] * omc, n[0] * n[2] * omc, n[1] * n[2] * omc
            R = [[n[0] * n[0] * omc + cs, xy + n[2] * sn, xz - n[1] * sn],
                 [xy - n[2] * sn, n[1] * n[1] * omc + cs, yz + n[0] * sn],
                 [xz + n[1] * sn, yz - n[0] * sn, n[2] * n[2] * omc + cs]]
            total, c = 0.0, [0.0, 0.0, 0.0]
            for a in range(lo, hi):
                total += masses[a]
                for k in range(3):
                    c[k] += masses[a] * pos[a][k]
            com = [c[k] / total for k in range(3)]
            new = pos[lo:hi].copy()
            for r, a in enumerate(range(lo, hi)):
                v = [pos[a][k] - com[k] for k in range(3)]
                new[r] = [com[k] + (R[k][0] * v[0] + R[k][1] * v[1] + R[k][2] * v[2]) for k in range(3)]
        u = rng.uniform()
        cost = beta * orc.move_molecule_cost(m, new)
        if cost <= 0.0 or u < math.exp(-cost):
            if not rotate:  # Molecule::wrap by the centre of mass
                total, c = 0.0, np.zeros(3)
                for r, a in enumerate(range(lo, hi)):
                    total += masses[a]
                    c = c + masses[a] * new[r]
                com = c / total
                new = new + (np.array(system.cell.wrap_vector(com)) - com)
            pos[lo:hi] = new
            orc.set_positions(pos)
            if refresh:
                orc.cache_init()
            else:
                orc.cache_update()
            accepted += 1
    return pos, orc.cache_energy(), accepted


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_molecular_chains_follow_the_oracle_move_for_move(precision):
    """Rigid 5-atom chains (LJ between molecules, Exclude13 inside them) with
    Translate and Rotate at equal frequency, next to a single-atom chain in
    the same batch, whose moves stay those of its own replay."""
    import systems as test_systems
    mol = test_systems.chains(27, 24.0, 3, lg.PairRestriction.EXCLUDE13)
    atoms = workloads.lj_replica(300, 0.6, 120.0, 11)
    batch = Batch([mol, atoms], precision=precision)
    batch.md_setup([1.0, 1.0])
    batch.mc_setup_moves(0, 300.0, translate=(0.3, 1.0), rotate=(0.15, 1.0), seed=41)
    batch.mc_setup(1, 120.0, 0.3, 100)
    moves = 300
    batch.mc_run(moves)
    mol_ref = test_systems.chains(27, 24.0, 3, lg.PairRestriction.EXCLUDE13)
    pos_ref, e_ref, acc_ref = replay_molecular(mol_ref, 300.0, 0.3, 1.0, 0.15, 1.0, 41, moves)
    energy, acc, att = batch.mc_stats(0)
    pos, _ = batch.state(0)
    assert att == moves and acc == acc_ref and 0 < acc < moves
    assert np.abs(pos - pos_ref).max() < 1e-9
    assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)
    pos_a, e_a, acc_a = replay(workloads.lj_replica(300, 0.6, 120.0, 11), 120.0, 0.3, 100, moves)
    energy, acc, att = batch.mc_stats(1)
    pos, _ = batch.state(1)
    assert acc == acc_a and np.abs(pos - pos_a).max() < 1e-9


@pytest.mark.parametrize("coulomb", ["wolf", "ewald"])
def test_molecular_chains_with_coulomb_follow_the_oracle(coulomb):
    """Charged rigid chains with Wolf or Ewald: the chain adds the real-space
    Coulomb terms of the moved molecule's neighbours and, for Ewald, the
    k-space change from delta rho(k), which an accepted move adds to rho(k)."""
    import systems as test_systems

    def make():
        c = {"wolf": lg.Wolf(8.0), "ewald": lg.Ewald(9.0, 5, 0.35)}[coulomb]
        return test_systems.chains(27, 24.0, 5, lg.PairRestriction.INTER_MOLECULAR, coulomb=c)
    s = make()
    batch = Batch([s])
    batch.md_setup([1.0])
    batch.mc_setup_moves(0, 300.0, translate=(0.3, 1.0), rotate=(0.15, 1.0), seed=43)
    moves = 200
    batch.mc_run(moves)
    pos_ref, e_ref, acc_ref = replay_molecular(make(), 300.0, 0.3, 1.0, 0.15, 1.0, 43, moves,
                                               refresh=coulomb == "ewald")
    energy, acc, att = batch.mc_stats(0)
    pos, _ = batch.state(0)
    assert att == moves and acc == acc_ref and acc > 0
    assert np.abs(pos - pos_ref).max() < 1e-9
    assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)
    assert abs(energy - batch.energy(0)) <= 1e-9 * abs(e_ref)  # the chain's energy is the fresh energy


def test_single_atom_chains_with_ewald_run_in_the_molecular_kernel():
    """lg_mc_setup of a system with Coulomb interactions (NaCl, Ewald): one-ion
    molecules through the molecular chains' kernel."""
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    batch = Batch([s])
    batch.md_setup([1.0])
    batch.mc_setup(0, 300.0, 0.3, 9)
    batch.mc_run(200)
    pos_ref, e_ref, acc_ref = replay_molecular(workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5), 300.0, 0.3,
                                               1.0, 0.0, 0.0, 9, 200, refresh=True)
    energy, acc, att = batch.mc_stats(0)
    pos, _ = batch.state(0)
    assert acc == acc_ref and np.abs(pos - pos_ref).max() < 1e-9
    assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)
