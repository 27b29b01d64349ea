"""Mixed precision against the FP64 oracle.

Stated tolerances of the mixed path (FP32 pair / Ewald arithmetic, compensated
FP32 force sums, FP64 energies, virials, rho(k) and state):
  relative force RMS error    <= 1e-5
  relative energy error       <= 1e-6
  virial (relative to max)    <= 1e-5
"""
import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu

F_TOL, E_TOL, W_TOL = 1e-5, 1e-6, 1e-5


def errors(system):
    orc = oracle.Oracle(system)
    f, e, w = system.compute()
    fo, eo, wo = orc.forces(), orc.energy(), orc.virial()
    ferr = np.sqrt(np.mean((f - fo) ** 2)) / np.sqrt(np.mean(fo ** 2))
    return ferr, abs(e - eo) / abs(eo), np.abs(w - wo).max() / np.abs(wo).max()


def check(system):
    ferr, eerr, werr = errors(system)
    assert ferr <= F_TOL, ferr
    assert eerr <= E_TOL, eerr
    assert werr <= W_TOL, werr


def test_mixed_argon():
    s = workloads.argon_fcc(precision="mixed")
    rng = np.random.default_rng(1)
    s.positions = s.positions + rng.uniform(-0.3, 0.3, size=s.positions.shape)
    check(s)


def test_mixed_nacl_ewald():
    check(workloads.nacl_crystal(precision="mixed"))


def test_mixed_nacl_wolf():
    check(workloads.nacl_crystal(precision="mixed", coulomb="wolf"))


def test_mixed_water():
    s = workloads.water_box(n_side=7, length=21.76, precision="mixed")
    rng = np.random.default_rng(2)
    s.positions = s.positions + rng.uniform(-0.05, 0.05, size=s.positions.shape)
    check(s)


@pytest.mark.parametrize("family", ["buckingham", "bmh", "morse", "gaussian", "mie", "table"])
def test_mixed_unwrapped_fluid(family):
    check(systems.random_lj_fluid(700, 0.02, 5, 9.0, family=family, precision="mixed"))


def test_mixed_chains_with_dihedrals():
    s = systems.chains(27, 24.0, 9, lg.PairRestriction.EXCLUDE13, coulomb=lg.Wolf(8.0), dihedrals=True)
    s.precision = "mixed"  # (before the engine is created)
    check(s)


def test_mixed_md_tracks_fp64():
    """Short trajectories of the two precisions stay within 1e-6 A."""
    a = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    b = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5, precision="mixed")
    for s in (a, b):
        md = lg.MolecularDynamics(lg.VelocityVerlet(1.0))
        md.setup(s)
        md.run(s, 20)
    assert np.abs(a.positions - b.positions).max() < 1e-6
