"""The benchmark configurations themselves, at their stated sizes, against the
FP64 oracle.

* The SPC/E-geometry water box at full size: 1728 molecules (5184 atoms) in a
  37.3 A cell, Ewald alpha 0.3 / kmax 8 (1051 k-vectors) / rc 10 A with the
  InterMolecular restriction (excluded intramolecular pairs take the -erf
  correction, lumol-core/src/energy/global/ewald.rs:394-397), O-O LJ at 10 A,
  harmonic bonds and angles.  FP64: forces, energy and virial of every term
  within 1e-10 (sys/compute.rs:30-255), pair sets bit for bit; mixed: the
  mixed path's stated tolerances (forces 1e-5 RMS, energy 1e-6, virial 1e-5).
* A sample of the batched-replica shapes: the smallest legal boxes (N = 64 at
  rho* = 0.5 and N = 113 at rho* = 0.9, three cells of the list radius per
  axis, where the cell stencil wraps onto itself), the largest, sparsest
  replica (N = 4096 at rho* = 0.3) and a mid-size one.  FP64 forces, energy
  and virial at 1e-10; 50 FP64 Velocity-Verlet + Berendsen steps against the
  oracle's trajectory (lumol-sim/src/md/integrators.rs:22-70,
  md/thermostats.rs:112-121) at 1e-9 A; the mixed per-step and persistent-
  kernel trajectories against the same FP64 oracle trajectory at 1e-6 A.
"""
import numpy as np
import pytest

import lumol_gb300 as lg
from lumol_gb300.batch import Batch
import oracle
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10
F_TOL, E_TOL, W_TOL = 1e-5, 1e-6, 1e-5
TERMS = [lg.LG_TERM_ALL, lg.LG_TERM_PAIRS, lg.LG_TERM_BONDS, lg.LG_TERM_ANGLES, lg.LG_TERM_COUL_REAL,
         lg.LG_TERM_COUL_SELF, lg.LG_TERM_COUL_KSPACE]


def _errors(f, e, w, fo, eo, wo):
    frms = np.sqrt(np.mean(fo * fo))
    ferr = np.sqrt(np.mean((f - fo) ** 2)) / frms if frms > 0 else float(np.abs(f).max())
    return ferr, abs(e - eo) / max(abs(eo), 1e-300), np.abs(w - wo).max() / max(np.abs(wo).max(), 1e-300)


@pytest.fixture(scope="module")
def water_full():
    s = workloads.water_box()  # 12^3 molecules, L = 37.3, kmax 8, alpha 0.3, rc 10, InterMolecular
    rng = np.random.default_rng(21)
    s.positions = s.positions + rng.uniform(-0.05, 0.05, size=s.positions.shape)
    return s


def test_water_full_size_fp64(water_full):
    s = water_full
    assert s.size == 5184
    orc = oracle.Oracle(s)
    for terms in TERMS:
        f, e, w = s.compute(terms)
        fo, eo, wo = orc.forces(terms), orc.energy(terms), orc.virial(terms)
        ferr, eerr, werr = _errors(f, e, w, fo, eo, wo)
        assert ferr <= TOL and eerr <= TOL and werr <= TOL, (terms, ferr, eerr, werr)
    for family in (0, 1):
        gpu, ref = s.pair_set(family), orc.pairset(family)
        assert gpu.shape == ref.shape and np.array_equal(gpu, ref), family


def test_water_full_size_mixed(water_full):
    s = water_full
    m = workloads.water_box(precision="mixed")
    m.positions = s.positions
    orc = oracle.Oracle(s)
    f, e, w = m.compute()
    ferr, eerr, werr = _errors(f, e, w, orc.forces(), orc.energy(), orc.virial())
    assert ferr <= F_TOL and eerr <= E_TOL and werr <= W_TOL, (ferr, eerr, werr)


REPLICAS = [(64, 0.5, 120.0), (113, 0.9, 95.0), (4096, 0.3, 280.0), (1500, 0.6, 200.0)]


def _replica(k, precision="fp64"):
    n, rho, t = REPLICAS[k]
    return workloads.lj_replica(n, rho, t, seed=500 + k, precision=precision)


@pytest.mark.parametrize("k", range(len(REPLICAS)))
def test_replica_shapes_fp64_forces(k):
    s = _replica(k)
    n, rho, _ = REPLICAS[k]
    L = s.cell.lengths[0]
    assert 0.5 * L >= 2.5 * 3.405  # a legal cutoff (sys/system.rs:122-131)
    orc = oracle.Oracle(s)
    for terms in (lg.LG_TERM_ALL, lg.LG_TERM_PAIRS):
        f, e, w = s.compute(terms)
        ferr, eerr, werr = _errors(f, e, w, orc.forces(terms), orc.energy(terms), orc.virial(terms))
        assert ferr <= TOL and eerr <= TOL and werr <= TOL, (terms, ferr, eerr, werr)
    gpu, ref = s.pair_set(0), orc.pairset(0)
    assert np.array_equal(gpu, ref)


def _oracle_trajectory(k, steps):
    s = _replica(k)
    orc = oracle.Oracle(s)
    n, rho, t = REPLICAS[k]
    xo, vo, _ = orc.velocity_verlet(s.positions, s.velocities, np.zeros((s.size, 3)), 1.0, steps, t, 100.0)
    return xo, vo


def test_replica_shapes_fp64_trajectories():
    """50 steps of VelocityVerlet + BerendsenThermostat(T, tau = 100 fs) of each
    replica, batched in one FP64 engine, against the oracle."""
    systems = [_replica(k) for k in range(len(REPLICAS))]
    batch = Batch(systems)
    batch.md_setup([1.0] * len(systems), thermostats=[(t, 100.0) for _, _, t in REPLICAS])
    batch.md_run(50)
    for k in range(len(REPLICAS)):
        x, v = batch.state(k)
        xo, vo = _oracle_trajectory(k, 50)
        assert np.abs(x - xo).max() < 1e-9, k
        assert np.abs(v - vo).max() / np.abs(vo).max() < 1e-8, k
    batch.engine.close()


@pytest.mark.parametrize("persistent", [False, True])
def test_replica_shapes_mixed_trajectories(persistent):
    """The same 24 steps on the mixed path, per-step kernels or one persistent
    launch, against the FP64 oracle trajectory at 1e-6 A."""
    systems = [_replica(k, "mixed") for k in range(len(REPLICAS))]
    batch = Batch(systems, precision="mixed", threads_per_atom=8, persistent=persistent)
    batch.md_setup([1.0] * len(systems), thermostats=[(t, 100.0) for _, _, t in REPLICAS])
    batch.md_run(24)
    cluster = ctypes_plan(batch)
    assert (cluster > 0) == persistent
    for k in range(len(REPLICAS)):
        x, v = batch.state(k)
        xo, vo = _oracle_trajectory(k, 24)
        assert np.abs(x - xo).max() < 1e-6, (k, np.abs(x - xo).max())
        assert np.abs(v - vo).max() / np.abs(vo).max() < 1e-5, k
    batch.engine.close()


def ctypes_plan(batch):
    import ctypes
    c, g = ctypes.c_int32(), ctypes.c_int32()
    batch.engine.call("lg_md_plan", ctypes.byref(c), ctypes.byref(g))
    return c.value
