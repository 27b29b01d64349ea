"""The Berendsen barostats (lumol-sim/src/md/integrators.rs:174-342) on the GPU
against the oracle's restatement.

FP64: positions within 1e-9 A and cell lengths within 1e-12 relative of the
oracle after every run, for LJ argon (cells of the list grid change as the
box shrinks: the batch is lowered again in place) and for NaCl with Ewald
(the k-vector factors follow the cell at every step); the mixed path within
1e-6 A.  A compression below twice the cutoff fails with the reference's
panic message.  The anisotropic barostat likewise (positions 1e-9 A, the
cell matrix 1e-12), from an orthorhombic cell (which keeps its shape and
takes off-diagonal terms) and from a triclinic one with a full stress
target.
"""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
from lumol_gb300 import _capi as C
from lumol_gb300 import units, workloads

pytestmark = pytest.mark.gpu


def _pressure(system):
    """System::pressure at the system's positions and velocities (compute.rs:399-431)."""
    from lumol_gb300.units import K_BOLTZMANN
    w = system.compute(C.LG_TERM_ALL, C.LG_WANT_VIRIAL)[2]
    dof = 3 * system.size
    T = 2.0 * system.kinetic_energy() / (dof * K_BOLTZMANN)
    return (dof * K_BOLTZMANN * T + np.trace(w)) / (3.0 * system.cell.volume())


def _run(make, precision, pressure, tau, runs):
    s = make(precision)
    ref = make("fp64")
    orc = oracle.Oracle(ref)
    md = lg.MolecularDynamics(lg.BerendsenBarostat(1.0, pressure, tau))
    md.setup(s)
    x, v, a, eta = ref.positions.copy(), ref.velocities.copy(), np.zeros((ref.size, 3)), 1.0
    out = []
    for k in runs:
        md.run(s, k)
        x, v, a, eta, cell = orc.berendsen_barostat(x, v, a, eta, 1.0, pressure, tau, k)
        out.append((s.positions.copy(), s.velocities.copy(), np.array(s.cell.lengths), x, v, cell))
    return out


@pytest.mark.parametrize("precision,tol,cell_tol", [("fp64", 1e-9, 1e-12), ("mixed", 1e-6, 1e-7)])
def test_barostat_argon_compression_changes_the_cell_grid(precision, tol, cell_tol):
    """(The mixed path's pressure carries the FP32 pair virial's ~1e-6 relative
    error, hence its looser cell tolerance.)"""
    base = workloads.argon_fcc()
    target = _pressure(base) + units.from_(10000.0, "bar")  # compresses the box by ~5 % in 6 steps
    out = _run(lambda p: workloads.argon_fcc(precision=p), precision, target, 30.0, [1, 2, 3, 5, 8])
    for x, v, cell, xo, vo, cello in out:
        assert np.abs(cell - cello).max() <= cell_tol * cello.max(), (cell, cello)
        assert np.abs(x - xo).max() < tol, np.abs(x - xo).max()
    # the box shrank through a change of the list's cell grid (5 -> 4 cells per
    # axis below 27.5 A, cells at least (rc + skin) / 2 = 5.5 A wide)
    assert out[-1][2][0] < 27.5, out[-1][2][0]


def test_barostat_nacl_ewald_follows_the_oracle():
    base = workloads.nacl_crystal(cells=4, cutoff=8.0, kmax=6)
    target = _pressure(base) - units.from_(2000.0, "bar")  # expands
    out = _run(lambda p: workloads.nacl_crystal(cells=4, cutoff=8.0, kmax=6, precision=p), "fp64", target,
               50.0, [4, 4, 8])
    for x, v, cell, xo, vo, cello in out:
        assert np.abs(cell - cello).max() <= 1e-12 * cello.max(), (cell, cello)
        assert np.abs(x - xo).max() < 1e-9, np.abs(x - xo).max()
        assert np.abs(v - vo).max() / np.abs(vo).max() < 1e-8


def test_barostat_below_twice_the_cutoff_fails_like_the_reference():
    s = workloads.argon_fcc()
    md = lg.MolecularDynamics(lg.BerendsenBarostat(1.0, units.from_(1e8, "bar"), 1.0))
    md.setup(s)
    with pytest.raises(lg.EngineError, match="Tried to decrease the cell size in Berendesen barostat"):
        md.run(s, 20)


def test_barostat_needs_velocity_verlet():
    s = workloads.argon_fcc()
    eng = s.engine()
    p = lg.md_params(lg.Verlet(1.0))
    eng.call("lg_md_setup_ex", 0, ctypes.byref(p))
    with pytest.raises(lg.EngineError):
        eng.call("lg_md_set_barostat", 0, C.LG_BAROSTAT_BERENDSEN, 0.0, 10.0)


# ---- AnisoBerendsenBarostat (integrators.rs:252-342) ----------------------------------
def _aniso_run(make, stress, tau, runs, precision="fp64"):
    s = make(precision)
    ref = make("fp64")
    orc = oracle.Oracle(ref)
    md = lg.MolecularDynamics(lg.AnisoBerendsenBarostat(1.0, stress, tau))
    md.setup(s)
    x, v, a, eta = ref.positions.copy(), ref.velocities.copy(), np.zeros((ref.size, 3)), np.eye(3)
    out = []
    for k in runs:
        md.run(s, k)
        x, v, a, eta, cell = orc.aniso_barostat(x, v, a, eta, 1.0, stress, tau, k)
        out.append((s.positions.copy(), s.velocities.copy(), s.cell.matrix(), s.cell.shape, x, v, cell))
    return out


def _replica(precision):
    return workloads.lj_replica(500, 0.6, 200.0, seed=4, precision=precision)


def test_aniso_barostat_hydrostatic_follows_the_oracle():
    """An orthorhombic cell takes off-diagonal terms (cell * eta with a
    symmetric eta) and keeps its shape; the orthorhombic branches then read
    its diagonal, the k-vectors and face distances the whole matrix."""
    stress = units.from_(1e4, "bar") * np.eye(3)
    for x, v, cell, shape, xo, vo, co in _aniso_run(_replica, stress, 100.0, [1, 3, 8]):
        assert np.abs(x - xo).max() < 1e-9, np.abs(x - xo).max()
        assert np.abs(v - vo).max() / np.abs(vo).max() < 1e-8
        assert np.abs(cell - co).max() <= 1e-12 * np.abs(co).max()
        assert shape == "orthorhombic"
    off = np.abs(cell - np.diag(np.diag(cell))).max()
    assert off > 0.0  # the cell is no longer diagonal


def test_aniso_barostat_stress_target_on_a_triclinic_cell():
    stress = units.from_(1.0, "bar") * np.array([[2e3, 3e2, 0.0], [3e2, 1e3, -2e2], [0.0, -2e2, 5e2]])

    def make(precision):
        s = _replica(precision)
        L = np.array(s.cell.lengths)
        cell = lg.UnitCell.triclinic(L[0], L[1], L[2], 85.0, 95.0, 100.0)
        frac = s.positions / L
        s.cell = cell
        s.positions = frac @ cell.matrix().T
        return s
    for x, v, cell, shape, xo, vo, co in _aniso_run(make, stress, 100.0, [2, 6]):
        assert np.abs(x - xo).max() < 1e-9, np.abs(x - xo).max()
        assert np.abs(cell - co).max() <= 1e-12 * np.abs(co).max()
        assert shape == "triclinic"


def test_aniso_barostat_mixed_precision_tracks_fp64():
    stress = units.from_(1e4, "bar") * np.eye(3)
    for x, v, cell, shape, xo, vo, co in _aniso_run(_replica, stress, 100.0, [1, 3, 8], precision="mixed"):
        assert np.abs(x - xo).max() < 1e-6, np.abs(x - xo).max()
        assert np.abs(cell - co).max() <= 1e-7 * np.abs(co).max()


def test_aniso_barostat_below_twice_the_cutoff_fails_like_the_reference():
    s = workloads.argon_fcc()
    md = lg.MolecularDynamics(lg.AnisoBerendsenBarostat.hydrostatic(1.0, units.from_(1e8, "bar"), 1.0))
    md.setup(s)
    with pytest.raises(lg.EngineError, match="Tried to decrease the cell size in anisotropic Berendesen barostat"):
        md.run(s, 20)
