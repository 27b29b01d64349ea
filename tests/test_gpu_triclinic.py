"""Triclinic cells on the GPU (UnitCell::triclinic, cells.rs:72-94; the
triclinic branches of vector_image / wrap_vector, cells.rs:263-301; the
general k-vectors of compute_ewald_factors_triclinic, ewald.rs:130-183),
against the oracle.

Bars as for orthorhombic cells: FP64 pair sets bit for bit, energies /
forces / virials within 1e-10, trajectories within 1e-9 A (velocity-Verlet
runs long enough to rebuild the lists in the fractional cell grid); the
mixed path within its stated tolerances (forces 1e-5, energy 1e-6, virial
1e-5) and 1e-6 A over 20 steps; Monte Carlo costs within 1e-10 of the
energy; the barostat's cell matrix within 1e-12.  The cell geometry the
engine derives (face distances, volume) equals the oracle's bit for bit."""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import _capi as C
from lumol_gb300 import units, workloads
from test_gpu_mixed import check as mixed_check
from test_gpu_parity import _pairset_equal, assert_parity, jitter

pytestmark = pytest.mark.gpu

ANGLES = (80.0, 95.0, 105.0)


def to_triclinic(s, angles=ANGLES, stretch=(1.04, 1.0, 0.97)):
    """The same fractional coordinates (unwrapped: whole cell vectors kept) in
    a triclinic cell of about the same lengths."""
    L = np.array(s.cell.lengths)
    cell = lg.UnitCell.triclinic(L[0] * stretch[0], L[1] * stretch[1], L[2] * stretch[2], *angles)
    frac = s.positions / L
    s.cell = cell
    s.positions = frac @ cell.matrix().T
    rc = max([p.cutoff for p in s.pairs.values()] + [s.coulomb.cutoff if s.coulomb else 0.0])
    assert min(cell.lengths) > 2.0 * rc, (cell.lengths, rc)
    return s


def nacl(coulomb="ewald", precision="fp64"):
    return to_triclinic(workloads.nacl_crystal(cells=5, precision=precision, coulomb=coulomb))


def water(precision="fp64"):
    s = workloads.water_box(n_side=7, length=24.0, precision=precision, cutoff=9.0, kmax=6)
    return to_triclinic(jitter(s, 0.05, 2))


def fluid(precision="fp64", n=700, seed=5):
    return to_triclinic(systems.random_lj_fluid(n, 0.02, seed, 9.0, family="lj", precision=precision))


# ---- energies, forces, virials and pair sets (FP64) ---------------------------------
@pytest.mark.parametrize("make", [
    lambda: to_triclinic(jitter(workloads.argon_fcc(), 0.3, 1)),
    lambda: nacl("ewald"),
    lambda: nacl("wolf"),
    lambda: water(),
    lambda: fluid(),
], ids=["argon", "nacl_ewald", "nacl_wolf", "water_ewald_bonds", "unwrapped_fluid"])
def test_fp64_parity(make):
    assert_parity(make())


def test_chains_restrictions_and_dihedrals():
    """Bond paths, angles and dihedral angles through the triclinic image."""
    s = to_triclinic(systems.chains(27, 24.0, 9, lg.PairRestriction.EXCLUDE13, coulomb=lg.Wolf(8.0),
                                    dihedrals=True), stretch=(1.1, 1.1, 1.1))
    assert_parity(s)


def test_pair_sets_bit_for_bit():
    _pairset_equal(nacl("ewald"))
    _pairset_equal(fluid(n=1500, seed=11))


def test_cell_geometry_matches_the_oracle():
    s = nacl("ewald")
    eng = s.engine()
    shape, lengths, volume = ctypes.c_int32(), np.zeros(3), ctypes.c_double()
    s.compute()
    eng.call("lg_cell_info", 0, ctypes.byref(shape), C.dptr(lengths), ctypes.byref(volume))
    ol, ov = oracle.Oracle(s).cell_info()
    assert shape.value == C.LG_CELL_TRICLINIC
    assert np.array_equal(lengths, ol) and volume.value == ov
    assert tuple(lengths) == s.cell.lengths and volume.value == s.cell.volume()
    m = np.zeros(9)
    eng.call("lg_get_cell", 0, C.dptr(m))
    assert np.array_equal(m, s.cell.matrix().ravel())


# ---- mixed precision ----------------------------------------------------------------
@pytest.mark.parametrize("make", [lambda: nacl("ewald", "mixed"), lambda: water("mixed"),
                                  lambda: fluid("mixed")], ids=["nacl_ewald", "water", "fluid"])
def test_mixed_precision_tolerances(make):
    mixed_check(make())


# ---- molecular dynamics ---------------------------------------------------------------
def test_velocity_verlet_through_list_rebuilds():
    """150 steps of 2 fs at 400 K: atoms move past half the skin, so the
    lists are rebuilt in the fractional cell grid several times."""
    s = fluid()
    s.velocities = workloads.boltzmann_velocities(s, 400.0, 3)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(2.0), lg.BerendsenThermostat(400.0, 50.0))
    md.setup(s)
    for k in (1, 49, 100):
        md.run(s, k)
    xo, vo, _ = orc.velocity_verlet(x0, v0, np.zeros_like(x0), 2.0, 150, 400.0, 50.0)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8
    assert np.abs(s.positions - x0).max() > 1.0  # the lists were rebuilt


def test_ewald_md_matches_the_oracle():
    s = to_triclinic(workloads.nacl_crystal(cells=3, cutoff=7.5, kmax=5), stretch=(1.1, 1.1, 1.1))
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0))
    md.setup(s)
    md.run(s, 25)
    xo, vo, _ = orc.velocity_verlet(x0, v0, np.zeros_like(x0), 1.0, 25)
    assert np.abs(s.positions - xo).max() < 1e-9


def test_rewrap_control_wraps_in_the_triclinic_cell():
    """Rewrap moves each molecule's centre of mass into the cell with
    wrap_vector's triclinic branch (controls.rs, molecules.rs:256-296)."""
    s = fluid(n=300, seed=8)
    s.velocities = workloads.boltzmann_velocities(s, 150.0, 9)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0), None, (lg.Rewrap,))
    md.setup(s)
    md.run(s, 20)
    p = lg.md_params(lg.VelocityVerlet(1.0), None, (lg.Rewrap,))
    xo, vo, _, _ = orc.md_run(x0, v0, np.zeros_like(x0), 20, integrator=0, dt=1.0, controls=p.controls)
    assert np.abs(s.positions - xo).max() < 1e-9
    frac = s.positions @ np.linalg.inv(s.cell.matrix()).T
    assert frac.min() > -1e-9 and frac.max() < 1.0 + 1e-9  # wrapped into the cell


def test_mixed_md_tracks_fp64_and_stays_off_the_persistent_kernel():
    from lumol_gb300.batch import Batch
    s = fluid("mixed")
    ref = fluid("fp64")
    b = Batch([s], precision="mixed")
    b.md_setup([1.0], [None])
    b.md_run(20)
    c, g = ctypes.c_int32(), ctypes.c_int32()
    b.engine.call("lg_md_plan", ctypes.byref(c), ctypes.byref(g))
    assert c.value <= 0  # the per-step kernels: the persistent kernel has no triclinic image
    x, _ = b.state(0)
    zeros = np.zeros((ref.size, 3))  # (the fluid starts at rest, as Batch.md_setup sets it up)
    xo, _, _ = oracle.Oracle(ref).velocity_verlet(ref.positions, zeros, zeros, 1.0, 20)
    assert np.abs(x - xo).max() < 1e-6
    b.engine.close()


def test_berendsen_barostat_scales_the_triclinic_cell():
    s = to_triclinic(workloads.lj_replica(500, 0.6, 200.0, seed=4), stretch=(1.0, 1.0, 1.0))
    ref = to_triclinic(workloads.lj_replica(500, 0.6, 200.0, seed=4), stretch=(1.0, 1.0, 1.0))
    orc = oracle.Oracle(ref)
    pressure = units.from_(1e4, "bar")
    md = lg.MolecularDynamics(lg.BerendsenBarostat(1.0, pressure, 30.0))
    md.setup(s)
    x, v, a, eta = ref.positions.copy(), ref.velocities.copy(), np.zeros((ref.size, 3)), 1.0
    for k in (1, 4, 10):
        md.run(s, k)
        x, v, a, eta, _ = orc.berendsen_barostat(x, v, a, eta, 1.0, pressure, 30.0, k)
        m = orc.cell_matrix()
        assert np.abs(s.positions - x).max() < 1e-9
        assert np.abs(s.cell.matrix() - m).max() <= 1e-12 * np.abs(m).max()
        assert s.cell.shape == "triclinic"
    assert not np.allclose(s.cell.matrix(), ref.cell.matrix())


# ---- Monte Carlo ------------------------------------------------------------------------
@pytest.mark.parametrize("coulomb", ["ewald", "wolf"])
def test_move_costs_match_the_oracle(coulomb):
    s = to_triclinic(systems.chains(27, 24.0, 3, lg.PairRestriction.INTER_MOLECULAR,
                                    coulomb={"ewald": lg.Ewald(9.0, 5, 0.35), "wolf": lg.Wolf(9.0)}[coulomb]),
                     stretch=(1.1, 1.1, 1.1))
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = s.mc_init()
    assert abs(e0 - orc.cache_energy()) <= 1e-10 * abs(e0)
    rng = np.random.default_rng(5)
    for molid in (3, 11, 20):
        lo, hi = s.molecule_range(molid)
        newpos = s.positions[lo:hi] + rng.uniform(-0.5, 0.5, size=3)
        cost = s.move_molecule_cost(molid, newpos)
        assert abs(cost - orc.move_molecule_cost(molid, newpos)) <= 1e-10 * abs(e0)
        wrapped = s.wrap_molecule(molid, newpos)
        e_gpu = s.mc_update(molid, wrapped)
        orc.set_positions(s.positions.copy())
        orc.cache_update()
        assert abs(e_gpu - orc.cache_energy()) <= 1e-9 * abs(e0)


def test_resize_costs_match_the_oracle():
    s = to_triclinic(workloads.lj_replica(400, 0.5, 150.0, seed=3), stretch=(1.0, 1.0, 1.0))
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = s.mc_init()
    eng = s.engine()
    cell, pos = s.cell, s.positions.copy()
    for factor, accept in [(1.03, True), (0.97, False), (0.985, True)]:
        new = cell.scaled(float(np.cbrt(factor)))
        newpos = pos.copy()
        for mol in range(int(s.molecules[-1]) + 1):
            lo, hi = s.molecule_range(mol)
            com = pos[lo:hi].mean(axis=0)
            newpos[lo:hi] = pos[lo:hi] + (np.array(new.cartesian(cell.fractional(com))) - com)
        c = ctypes.c_double()
        eng.call("lg_mc_move_all_molecules_cost", 0, C.dptr(np.ascontiguousarray(new.matrix().ravel())),
                 C.dptr(np.ascontiguousarray(newpos)), ctypes.byref(c))
        assert abs(c.value - orc.move_all_molecules_cost(new.matrix(), newpos)) <= 1e-10 * abs(e0)
        if accept:
            eng.call("lg_mc_update", 0, None, ctypes.byref(ctypes.c_double()))
            orc.cache_update()
            cell, pos = new, newpos
        else:
            eng.call("lg_mc_restore", 0)
            orc.cache_restore()
    m = np.zeros(9)
    eng.call("lg_get_cell", 0, C.dptr(m))
    assert np.array_equal(m, cell.matrix().ravel())


# ---- errors -------------------------------------------------------------------------------
def test_shape_and_chain_errors():
    s = nacl("ewald")
    eng = s.engine()
    m = s.cell.matrix().ravel().copy()
    m[0] = -m[0]  # an orthorhombic matrix needs a positive diagonal
    with pytest.raises(lg.EngineError):
        eng.call("lg_set_cell_ex", 0, C.dptr(m), C.LG_CELL_ORTHORHOMBIC)
    with pytest.raises(lg.EngineError):
        eng.call("lg_set_cell_ex", 0, C.dptr(np.zeros(9)), C.LG_CELL_TRICLINIC)



def test_device_chains_in_a_triclinic_cell():
    """A chain of a triclinic system runs in the molecular chains' kernel
    (general image and wrap): replayed move for move through the oracle."""
    from lumol_gb300.batch import Batch
    from test_gpu_mc_chains import replay_molecular
    s = fluid(n=300, seed=8)
    b = Batch([s])
    b.md_setup([1.0])
    b.mc_setup(0, 150.0, 0.3, 17)
    b.mc_run(300)
    pos_ref, e_ref, acc_ref = replay_molecular(fluid(n=300, seed=8), 150.0, 0.3, 1.0, 0.0, 0.0, 17, 300)
    energy, acc, att = b.mc_stats(0)
    pos, _ = b.state(0)
    assert att == 300 and acc == acc_ref and acc > 0
    assert np.abs(pos - pos_ref).max() < 1e-9
    assert abs(energy - e_ref) <= 1e-9 * abs(e_ref)
    b.engine.close()
