"""Verlet and LeapFrog integrators, Rescale and CSVR thermostats, and the
RemoveTranslation and Rewrap controls on the GPU (lumol-sim/src/md), against
the oracle and the reference's own tests.

Bars: FP64 trajectories within 1e-9 A of the oracle (velocities 1e-8
relative) over 25 steps split across run boundaries; the mixed path within
1e-6 A of the FP64 oracle over 20 steps; the reference's literal tests exact
(controls) or within 1e-12 K (Rescale); CSVR's kinetic-energy mean and
variance within statistical bounds (the noise is this engine's own stream)."""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import workloads
from lumol_gb300.batch import Batch
from lumol_gb300.units import K_BOLTZMANN

pytestmark = pytest.mark.gpu

INTEGRATORS = {"vv": lg.VelocityVerlet, "verlet": lg.Verlet, "leapfrog": lg.LeapFrog}
KIND = {"vv": 0, "verlet": 1, "leapfrog": 2}

# (Verlet with Rewrap is left out: Rewrap moves x but not Verlet's x(t - dt),
# in the reference as here, so a wrapped atom then jumps a cell length a step.)
CASES = [  # integrator, thermostat, controls
    ("vv", "csvr", ("translation",)),
    ("verlet", None, ()),
    ("verlet", "berendsen", ("translation",)),
    ("leapfrog", "rescale", ("rewrap",)),
    ("leapfrog", "csvr", ()),
    ("vv", "rescale", ("translation", "rewrap")),
    ("vv", "berendsen", ("translation", "rotation")),
    ("leapfrog", None, ("rotation", "rewrap")),
]


def thermostat(name):
    return {None: None,
            "berendsen": lg.BerendsenThermostat(140.0, 20.0),
            "rescale": lg.RescaleThermostat(140.0, 1.0),
            "csvr": lg.CSVRThermostat(140.0, 10.0, seed=11)}[name]


def controls(names):
    return tuple({"translation": lg.RemoveTranslation, "rewrap": lg.Rewrap, "rotation": lg.RemoveRotation}[c]
                 for c in names)


def fluid(precision="fp64"):
    s = systems.random_lj_fluid(300, 0.02, 8, 9.0, family="lj", precision=precision)
    s.velocities = workloads.boltzmann_velocities(s, 150.0, 9)
    return s


def oracle_run(s, integrator, th, ctl, dt, nsteps):
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    state = orc.verlet_setup(x0, v0, dt) if integrator == "verlet" else np.zeros_like(x0)
    p = lg.md_params(INTEGRATORS[integrator](dt), thermostat(th), controls(ctl))
    x, v, _, _ = orc.md_run(x0, v0, state, nsteps, integrator=KIND[integrator], dt=dt, thermostat=p.thermostat,
                            temperature=p.temperature, tau=p.tau, tolerance=p.tolerance, seed=p.seed,
                            controls=p.controls)
    return x, v


@pytest.mark.parametrize("integrator,th,ctl", CASES)
def test_md_matches_oracle(integrator, th, ctl):
    s = fluid()
    xo, vo = oracle_run(s, integrator, th, ctl, 1.0, 25)
    md = lg.MolecularDynamics(INTEGRATORS[integrator](1.0), thermostat(th), controls(ctl))
    md.setup(s)
    for k in (1, 3, 21):  # run boundaries: the pending thermostat and controls are applied at each
        md.run(s, k)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8


@pytest.mark.parametrize("integrator,th,ctl", CASES[:4])
def test_mixed_md_tracks_fp64_oracle(integrator, th, ctl):
    s = fluid("mixed")
    xo, _ = oracle_run(s, integrator, th, ctl, 1.0, 20)
    md = lg.MolecularDynamics(INTEGRATORS[integrator](1.0), thermostat(th), controls(ctl))
    md.setup(s)
    md.run(s, 20)
    assert np.abs(s.positions - xo).max() < 1e-6


def test_md_with_dihedrals_matches_oracle():
    """VelocityVerlet with Berendsen on flexible chains with Torsion and
    CosineHarmonic dihedral angles: the FP64 trajectory follows the oracle."""
    s = systems.chains(27, 24.0, 9, lg.PairRestriction.EXCLUDE13, coulomb=lg.Wolf(8.0), dihedrals=True)
    s.velocities = workloads.boltzmann_velocities(s, 250.0, 4)
    xo, vo = oracle_run(s, "vv", "berendsen", (), 0.5, 25)
    md = lg.MolecularDynamics(lg.VelocityVerlet(0.5), thermostat("berendsen"))
    md.setup(s)
    md.run(s, 25)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8


def two_silver(x1, v):
    s = lg.System(lg.UnitCell.cubic(10.0))
    s.add_particles(["Ag", "Ag"], np.array([[0.0, 0.0, 0.0], x1]), masses=[107.8682, 107.8682])
    s.velocities = np.array(v, dtype=float)
    return s


def test_controls_literals():
    # controls.rs:95-107 (RemoveTranslation) and 125-131 (Rewrap), after one step without forces
    s = two_silver([1.0, 1.0, 1.0], [[1.0, 2.0, 0.0], [1.0, 0.0, 0.0]])
    lg.MolecularDynamics(lg.VelocityVerlet(1e-3), None, (lg.RemoveTranslation,)).run(s, 1)
    assert s.velocities.tolist() == [[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]]
    s = two_silver([15.0, 0.0, 0.0], [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    lg.MolecularDynamics(lg.VelocityVerlet(1.0), None, (lg.Rewrap,)).run(s, 1)
    assert s.positions.tolist() == [[0.0, 0.0, 0.0], [5.0, 0.0, 0.0]]
    # controls.rs:109-122 (RemoveRotation): a step of 1e-300 fs moves the atoms by
    # about 1e-300 A, which leaves terms of that size in the result
    s = two_silver([1.0, 0.0, 0.0], [[0.0, 1.0, 0.0], [0.0, -1.0, 2.0]])
    lg.MolecularDynamics(lg.VelocityVerlet(1e-300), None, (lg.RemoveRotation,)).run(s, 1)
    assert np.abs(s.velocities - [[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]]).max() < 1e-12


def helium_gas(n_side=10, temperature=300.0, seed=42):
    """lumol-sim/tests/thermostats.rs:14-31: helium on a 2 A grid, 20 A cell."""
    s = lg.System(lg.UnitCell.cubic(2.0 * n_side))
    grid = np.array([[i, j, k] for i in range(n_side) for j in range(n_side) for k in range(n_side)], float) * 2.0
    s.add_particles(["He"] * len(grid), grid)
    v = np.random.default_rng(seed).normal(size=grid.shape)
    v -= v.mean(axis=0)
    s.velocities = v
    v *= np.sqrt(temperature / s.temperature())
    s.velocities = v
    return s


def test_rescale_literals():
    # lumol-sim/tests/thermostats.rs:34-49
    s = helium_gas()
    assert abs(s.temperature() - 300.0) < 1e-12
    lg.MolecularDynamics(lg.VelocityVerlet(1.0), lg.RescaleThermostat(250.0, 100.0)).run(s, 1)
    assert abs(s.temperature() - 300.0) < 1e-12
    lg.MolecularDynamics(lg.VelocityVerlet(1.0), lg.RescaleThermostat(250.0, 10.0)).run(s, 1)
    assert abs(s.temperature() - 250.0) < 1e-12


def test_csvr_samples_the_canonical_kinetic_energy():
    """lumol-sim/tests/thermostats.rs:80-117 on the 1000-atom ideal gas: mean
    kinetic energy dof kT / 2 and variance dof (kT)^2 / 2.  20000 steps after
    200 of equilibration, one sample every 10 steps: mean within 1 %, variance
    within 15 % (about three standard errors)."""
    s = helium_gas()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0), lg.CSVRThermostat(250.0, 10.0, seed=5))
    md.run(s, 200)
    kinetic = []
    m = s.masses[:, None]
    for _ in range(2000):
        md.run(s, 10)
        kinetic.append(0.5 * float(np.sum(m * s.velocities ** 2)))
    dof, kT = 3 * s.size, K_BOLTZMANN * 250.0
    assert abs(np.mean(kinetic) / (dof * kT / 2.0) - 1.0) < 0.01
    assert abs(np.var(kinetic) / (dof * kT * kT / 2.0) - 1.0) < 0.15


def test_batch_of_propagators_matches_each_alone():
    """Systems with different integrators, thermostats and controls in one
    engine give their standalone trajectories bit for bit."""
    specs = [("vv", "berendsen", ("rewrap",)), ("verlet", "rescale", ()), ("leapfrog", "csvr", ("translation",))]

    def make(k):
        s = systems.random_lj_fluid(200 + 50 * k, 0.02, 20 + k, 9.0, family="lj")
        s.velocities = workloads.boltzmann_velocities(s, 150.0, 30 + k)
        return s

    def props(k):
        i, th, ctl = specs[k]
        return lg.MolecularDynamics(INTEGRATORS[i](1.0), thermostat(th), controls(ctl))

    batch = Batch([make(k) for k in range(3)], threads_per_atom=8)
    batch.md_setup(propagators=[props(k) for k in range(3)])
    batch.md_run(30)
    for k in range(3):
        alone = Batch([make(k)], threads_per_atom=8)
        alone.md_setup(propagators=[props(k)])
        alone.md_run(30)
        pa, va = batch.state(k)
        pb, vb = alone.state(0)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb), k
        alone.engine.close()
    batch.engine.close()


def test_setup_checks_mirror_reference_panics():
    """CSVRThermostat::from_rng's check (thermostats.rs:151-160) in the C ABI."""
    s = fluid()
    p = lg.md_params(lg.VelocityVerlet(1.0))
    p.thermostat, p.temperature, p.tau = 3, 300.0, 0.5
    with pytest.raises(lg.EngineError, match="larger than 1 in CSVR"):
        s.engine().call("lg_md_setup_ex", 0, ctypes.byref(p))
