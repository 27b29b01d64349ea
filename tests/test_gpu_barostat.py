"""The Berendsen barostat (lumol-sim/src/md/integrators.rs:174-250) on the GPU
against the oracle's restatement.

FP64: positions within 1e-9 A and cell lengths within 1e-12 relative of the
oracle after every run, for LJ argon (cells of the list grid change as the
box shrinks: the batch is lowered again in place) and for NaCl with Ewald
(the k-vector factors follow the cell at every step); the mixed path within
1e-6 A.  A compression below twice the cutoff fails with the reference's
panic message.
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
