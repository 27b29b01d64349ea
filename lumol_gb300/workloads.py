"""Seeded synthetic systems of the benchmark and parity workloads.

No dataset ships with these workloads: each builder places atoms on a lattice
(with seeded jitter or orientations) and draws velocities with a seeded
generator.  Shapes, sizes and parameters follow the workload definitions:

* argon_fcc   -- 5x5x5 FCC argon (500 atoms, L = 28.8 A), shifted LJ, rc = 10 A
* nacl_crystal -- 5x5x5 rock salt (1000 ions, a = 5.64 A), LJ (Lorentz-Berthelot
                  pairs written out explicitly, since Lumol has no mixing rules),
                  Ewald rc = 9 A, alpha = 0.35 / A, kmax = 7
* water_box   -- 12^3 SPC/E-geometry waters (5184 atoms, L = 37.3 A), harmonic
                  bonds and angles, O-O LJ, Ewald alpha = 0.3 / A, kmax = 8,
                  rc = 10 A, intermolecular restriction
"""
from __future__ import annotations

import math

import numpy as np

from .system import (Ewald, Harmonic, LennardJones, NullPotential, PairInteraction, PairRestriction,
                     System, UnitCell)
from .units import K_BOLTZMANN, from_


def boltzmann_velocities(system: System, temperature: float, seed: int) -> np.ndarray:
    """Maxwell-Boltzmann velocities with the post-processing of
    BoltzmannVelocities::init (lumol-sim/src/velocities.rs:56-66):
    RemoveTranslation, RemoveRotation (md/controls.rs:20-60), then a rescale to
    `temperature`.  The random stream is numpy's, seeded."""
    rng = np.random.default_rng(seed)
    m = system.masses
    v = rng.normal(0.0, math.sqrt(K_BOLTZMANN * temperature), size=(system.size, 3))
    v *= np.sqrt(1.0 / m)[:, None]
    # RemoveTranslation
    total = m.sum()
    v -= (v * m[:, None] / total).sum(axis=0)
    # RemoveRotation
    x = system.positions
    com = (x * m[:, None]).sum(axis=0) / total
    d = x - com
    moment = (m[:, None] * np.cross(d, v)).sum(axis=0)
    inertia = -(m[:, None, None] * d[:, :, None] * d[:, None, :]).sum(axis=0)
    inertia += np.eye(3) * np.trace(inertia)
    angular = np.linalg.solve(inertia, moment)
    v -= np.cross(d, angular)
    # velocities::scale
    kinetic = 0.5 * float((m[:, None] * v * v).sum())
    t_now = 2.0 * kinetic / (3 * system.size * K_BOLTZMANN)
    v *= math.sqrt(temperature / t_now)
    return v


def argon_fcc(cells: int = 5, a: float = 5.76, temperature: float = 300.0, seed: int = 0,
              precision: str = "fp64", cutoff: float = 10.0) -> System:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    grid = np.array([[i, j, k] for i in range(cells) for j in range(cells) for k in range(cells)], dtype=float)
    pos = ((grid[:, None, :] + base[None, :, :]).reshape(-1, 3)) * a
    system = System(UnitCell.cubic(cells * a), precision=precision)
    system.add_particles(["Ar"] * len(pos), pos, masses=[39.948] * len(pos))
    lj = LennardJones(sigma=3.405, epsilon=from_(0.996, "kJ/mol"))
    system.set_pair_potential(("Ar", "Ar"), PairInteraction.shifted(lj, cutoff))
    system.velocities = boltzmann_velocities(system, temperature, seed)
    return system


def nacl_crystal(cells: int = 5, a: float = 5.64, jitter: float = 0.05, seed: int = 0,
                 precision: str = "fp64", cutoff: float = 9.0, alpha: float = 0.35, kmax: int = 7,
                 temperature: float = 300.0, coulomb: str = "ewald") -> System:
    rng = np.random.default_rng(seed)
    na = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cl = na + np.array([0.5, 0.0, 0.0])
    names, pos = [], []
    for i in range(cells):
        for j in range(cells):
            for k in range(cells):
                for s in na:
                    names.append("Na")
                    pos.append((np.array([i, j, k]) + s) * a)
                for s in cl:
                    names.append("Cl")
                    pos.append((np.array([i, j, k]) + s) * a)
    pos = np.array(pos) + rng.uniform(-jitter, jitter, size=(len(pos), 3))
    charges = [1.0 if nm == "Na" else -1.0 for nm in names]
    system = System(UnitCell.cubic(cells * a), precision=precision)
    system.add_particles(names, pos, charges=charges)
    eps_na, eps_cl = from_(0.544, "kJ/mol"), from_(0.4184, "kJ/mol")
    system.set_pair_potential(("Na", "Na"), PairInteraction(LennardJones(2.35, eps_na), cutoff))
    system.set_pair_potential(("Cl", "Cl"), PairInteraction(LennardJones(4.40, eps_cl), cutoff))
    mixed = LennardJones(0.5 * (2.35 + 4.40), math.sqrt(eps_na * eps_cl))
    system.set_pair_potential(("Na", "Cl"), PairInteraction(mixed, cutoff))
    if coulomb == "ewald":
        system.set_coulomb_potential(Ewald(cutoff, kmax, alpha))
    elif coulomb == "wolf":
        from .system import Wolf
        system.set_coulomb_potential(Wolf(cutoff))
    system.velocities = boltzmann_velocities(system, temperature, seed + 1)
    return system


def _random_rotations(rng, n):
    # uniform quaternions (Shoemake)
    u1, u2, u3 = rng.random((3, n))
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    x, y, z, w = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], axis=1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], axis=1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1),
    ], axis=1)


def water_box(n_side: int = 12, length: float = 37.3, seed: int = 0, precision: str = "fp64",
              cutoff: float = 10.0, alpha: float = 0.3, kmax: int = 8, temperature: float = 300.0) -> System:
    rng = np.random.default_rng(seed)
    theta = math.radians(109.47)
    local = np.array([[0.0, 0.0, 0.0],
                      [1.0, 0.0, 0.0],
                      [math.cos(theta), math.sin(theta), 0.0]])
    spacing = length / n_side
    rot = _random_rotations(rng, n_side ** 3)
    system = System(UnitCell.cubic(length), precision=precision)
    m = 0
    for i in range(n_side):
        for j in range(n_side):
            for k in range(n_side):
                center = (np.array([i, j, k]) + 0.5) * spacing
                xyz = center + local @ rot[m].T
                system.add_molecule(["O", "H", "H"], xyz, bonds=[(0, 1), (0, 2)],
                                    charges=[-0.8476, 0.4238, 0.4238])
                m += 1
    system.set_pair_potential(("O", "O"), PairInteraction(LennardJones(3.166, from_(0.650, "kJ/mol")), cutoff))
    system.set_pair_potential(("O", "H"), PairInteraction(NullPotential(), cutoff))
    system.set_pair_potential(("H", "H"), PairInteraction(NullPotential(), cutoff))
    system.set_bond_potential(("O", "H"), Harmonic(k=from_(4637.0, "kJ/mol/A^2"), x0=1.0))
    system.set_angle_potential(("H", "O", "H"), Harmonic(k=from_(383.0, "kJ/mol/rad^2"), x0=theta))
    ewald = Ewald(cutoff, kmax, alpha)
    ewald.set_restriction(PairRestriction.INTER_MOLECULAR)
    system.set_coulomb_potential(ewald)
    system.velocities = boltzmann_velocities(system, temperature, seed + 1)
    return system


def lj_replica(n: int, reduced_density: float, temperature: float, seed: int, precision: str = "fp64",
               sigma: float = 3.405, epsilon_kj: float = 0.996) -> System:
    """One argon-type replica: `n` atoms on a jittered simple-cubic lattice at
    reduced density rho* = rho sigma^3, the argon workload's LJ parameters and
    energy-shifted cutoff (PairInteraction::shifted) at rc = 2.5 sigma,
    Maxwell-Boltzmann velocities at `temperature`."""
    rng = np.random.default_rng(seed)
    length = (n * sigma ** 3 / reduced_density) ** (1.0 / 3.0)
    side = int(math.ceil(n ** (1.0 / 3.0)))
    spacing = length / side
    grid = np.array([[i, j, k] for i in range(side) for j in range(side) for k in range(side)], dtype=float)
    grid = grid[rng.permutation(len(grid))[:n]]
    pos = (grid + 0.5) * spacing + rng.uniform(-0.1, 0.1, size=(n, 3)) * spacing
    system = System(UnitCell.cubic(length), precision=precision)
    system.add_particles(["Ar"] * n, pos, masses=[39.948] * n)
    lj = LennardJones(sigma=sigma, epsilon=from_(epsilon_kj, "kJ/mol"))
    system.set_pair_potential(("Ar", "Ar"), PairInteraction.shifted(lj, 2.5 * sigma))
    system.velocities = boltzmann_velocities(system, temperature, seed + 7)
    return system


def lj_replica_parameters(count: int = 256, seed: int = 2024, sigma: float = 3.405):
    """Seeded draws of the batched-replica workload: N ~ U{64..4096}, rho* ~
    U(0.3, 0.9), T ~ U(90, 300) K.  Draws whose box would be shorter than twice
    the cutoff (N < 125 rho*, where Lumol refuses the cutoff, sys/system.rs:122-131)
    are drawn again; the number of redraws is returned."""
    rng = np.random.default_rng(seed)
    params, redraws = [], 0
    while len(params) < count:
        n = int(rng.integers(64, 4097))
        rho = float(rng.uniform(0.3, 0.9))
        t = float(rng.uniform(90.0, 300.0))
        length = (n * sigma ** 3 / rho) ** (1.0 / 3.0)
        if 0.5 * length < 2.5 * sigma:
            redraws += 1
            continue
        params.append((n, rho, t))
    return params, redraws


def lj_replicas(count: int = 256, seed: int = 2024, precision: str = "fp64"):
    params, redraws = lj_replica_parameters(count, seed)
    systems = [lj_replica(n, rho, t, seed + 1000 + i, precision) for i, (n, rho, t) in enumerate(params)]
    return systems, params, redraws


def lj_fluid_like_argon(n: int, seed: int, precision: str = "fp64") -> System:
    """LJ fluid like the argon workload: `n` atoms at its density (500 / 28.8^3),
    jittered simple-cubic placement, shifted LJ, rc = 10 A."""
    density = 500.0 / 28.8 ** 3
    sigma = 3.405
    system = lj_replica(n, density * sigma ** 3, 300.0, seed, precision)
    lj = LennardJones(sigma=sigma, epsilon=from_(0.996, "kJ/mol"))
    system.pairs.clear()
    system.set_pair_potential(("Ar", "Ar"), PairInteraction.shifted(lj, 10.0))
    return system


def serving_requests(count: int = 48, rate: float = 40.0, seed: int = 77, precision: str = "mixed",
                     scale: float = 1.0):
    """Seeded request stream of the serving workload: Poisson arrivals at `rate`
    per second; 60 % LJ fluids like the argon workload (200-20000 atoms), 25 %
    NaCl Ewald crystals like the NaCl workload (3^3..10^3 conventional cells,
    216-8000 ions; rc = min(9 A, L/2)), 15 % water boxes like the water workload
    (300-3000 molecules); 500-5000 MD steps each.  `scale` < 1 shrinks sizes and
    step counts for tests."""
    from .serving import Request
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += float(rng.exponential(1.0 / rate))
        u = float(rng.random())
        steps = max(10, int(rng.integers(500, 5001) * scale))
        if u < 0.60:
            n = max(170, int(rng.integers(200, 20001) * scale))
            system, kind, dt = lj_fluid_like_argon(n, 3000 + rid, precision), "lj", 1.0
        elif u < 0.85:
            c = int(rng.integers(3, 11)) if scale >= 1.0 else int(rng.integers(3, 5))
            length = 5.64 * c
            rc = min(9.0, 0.5 * length * (1.0 - 1e-9))
            system, kind, dt = nacl_crystal(cells=c, cutoff=rc, precision=precision, seed=3000 + rid), "nacl", 1.0
        else:
            m = max(300, int(rng.integers(300, 3001) * scale))
            side = int(math.ceil(m ** (1.0 / 3.0)))
            length = 37.3 * (m / 1728.0) ** (1.0 / 3.0)
            system = water_box(n_side=side, length=length * side / m ** (1.0 / 3.0), precision=precision,
                               seed=3000 + rid)
            kind, dt = "water", 0.5
        out.append(Request(rid=rid, system=system, nsteps=steps, timestep=dt, arrival=t, kind=kind))
    return out
