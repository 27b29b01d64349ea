"""Parity of the FP64 GPU path with the CPU oracle, through the C ABI.

Bar: pair sets bit-for-bit; energies, virials and forces within 1e-10
relative (forces as the RMS of the difference over the RMS of the oracle's
forces; virials relative to their largest entry)."""
import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10
TERMS = [lg.LG_TERM_ALL, lg.LG_TERM_PAIRS, lg.LG_TERM_TAIL, lg.LG_TERM_BONDS, lg.LG_TERM_ANGLES,
         lg.LG_TERM_COUL_REAL, lg.LG_TERM_COUL_SELF, lg.LG_TERM_COUL_KSPACE, lg.LG_TERM_DIHEDRALS]


def _rel(a, b, scale):
    return abs(a - b) / max(abs(scale), 1e-300)


def assert_parity(system, terms_list=TERMS, tol=TOL):
    orc = oracle.Oracle(system)
    e_all = abs(orc.energy())
    for terms in terms_list:
        f, e, w = system.compute(terms)
        fo, eo, wo = orc.forces(terms), orc.energy(terms), orc.virial(terms)
        escale = max(abs(eo), 1e-12 * e_all, 1e-300)
        assert _rel(e, eo, escale) <= tol, (terms, e, eo)
        wscale = max(np.abs(wo).max(), 1e-300)
        assert np.abs(w - wo).max() / wscale <= tol or np.abs(wo).max() < 1e-14, (terms, w, wo)
        frms = np.sqrt(np.mean(fo * fo))
        if frms > 0:
            err = np.sqrt(np.mean((f - fo) ** 2)) / frms
            assert err <= tol, (terms, err)
        else:
            assert np.abs(f).max() == 0.0


def jitter(system, amount, seed):
    rng = np.random.default_rng(seed)
    system.positions = system.positions + rng.uniform(-amount, amount, size=system.positions.shape)
    return system


def test_argon_fcc_lj_shifted():
    s = jitter(workloads.argon_fcc(), 0.3, 1)
    assert_parity(s)


def test_nacl_ewald():
    s = workloads.nacl_crystal()
    assert_parity(s)


def test_nacl_wolf():
    s = workloads.nacl_crystal(coulomb="wolf")
    assert_parity(s)


def test_small_water_ewald_bonds_angles_exclusions():
    s = workloads.water_box(n_side=7, length=21.76)
    s = jitter(s, 0.05, 2)
    assert_parity(s)


def test_reference_unit_systems():
    s = systems.nacl_pair()
    s.set_coulomb_potential(lg.Ewald(8.0, 10))
    assert_parity(s)
    s = systems.ewald_water()
    ew = lg.Ewald(8.0, 10)
    ew.set_restriction(lg.PairRestriction.INTER_MOLECULAR)
    s.set_coulomb_potential(ew)
    assert_parity(s)
    assert_parity(systems.evaluator_system(), [lg.LG_TERM_PAIRS, lg.LG_TERM_TAIL, lg.LG_TERM_BONDS,
                                               lg.LG_TERM_ANGLES])


@pytest.mark.parametrize("family", ["lj", "buckingham", "bmh", "morse", "gaussian", "mie", "table"])
def test_two_kind_fluid_unwrapped(family):
    s = systems.random_lj_fluid(700, 0.02, 5, 9.0, family=family)
    assert_parity(s, [lg.LG_TERM_ALL, lg.LG_TERM_PAIRS, lg.LG_TERM_TAIL])


@pytest.mark.parametrize("restriction", [lg.PairRestriction.EXCLUDE12, lg.PairRestriction.EXCLUDE13,
                                         lg.PairRestriction.EXCLUDE14, lg.PairRestriction.scale14(0.5),
                                         lg.PairRestriction.INTRA_MOLECULAR])
def test_chain_restrictions_wolf(restriction):
    s = systems.chains(27, 24.0, 7, restriction, coulomb=lg.Wolf(8.0))
    assert_parity(s)


@pytest.mark.parametrize("restriction", [lg.PairRestriction.EXCLUDE13, lg.PairRestriction.INTER_MOLECULAR])
def test_chain_restrictions_ewald(restriction):
    s = systems.chains(27, 24.0, 8, restriction, coulomb=lg.Ewald(8.0, 6, 0.4))
    assert_parity(s)


@pytest.mark.parametrize("coulomb", [None, "wolf"])
def test_chain_dihedrals_and_cosine_angles(coulomb):
    """Torsion and CosineHarmonic dihedral angles and a CosineHarmonic angle
    (functions.rs:162-258; cells.rs:379-411; compute.rs:86-96)."""
    s = systems.chains(27, 24.0, 9, lg.PairRestriction.EXCLUDE13,
                       coulomb=lg.Wolf(8.0) if coulomb else None, dihedrals=True)
    assert len(s.dihedrals()) == 54
    assert_parity(s)


# ---- pair sets, bit for bit ----------------------------------------------------------
def _pairset_equal(system):
    orc = oracle.Oracle(system)
    for family in (0, 1):
        gpu = system.pair_set(family)
        ref = orc.pairset(family)
        assert gpu.shape == ref.shape and np.array_equal(gpu, ref), family


def test_pairset_nacl_and_water():
    _pairset_equal(workloads.nacl_crystal())
    _pairset_equal(jitter(workloads.water_box(n_side=7, length=21.76), 0.05, 3))


def test_pairset_atoms_exactly_at_cutoff():
    """Pairs at r == cutoff: excluded for pair potentials (r >= rc), kept by
    Ewald (r > rc is the test); and half-box separations for the image."""
    s = lg.System(lg.UnitCell.cubic(20.0))
    pos = [[0.0, 0.0, 0.0], [9.0, 0.0, 0.0], [0.0, 9.0, 0.0], [10.0, 10.0, 10.0], [3.0, 3.0, 3.0],
           [3.0, 3.0, 12.0], [-7.0, 3.0, 3.0], [1.5, 0.25, 19.0]]
    s.add_particles(["Na", "Cl"] * 4, pos, charges=[1.0, -1.0] * 4)
    for a, b in [("Na", "Na"), ("Na", "Cl"), ("Cl", "Cl")]:
        s.set_pair_potential((a, b), lg.PairInteraction(lg.LennardJones(2.5, 0.1), 9.0))
    s.set_coulomb_potential(lg.Ewald(9.0, 4, 0.3))
    _pairset_equal(s)
    assert_parity(s, [lg.LG_TERM_ALL])


def test_pairset_random_unwrapped_fluid():
    _pairset_equal(systems.random_lj_fluid(1500, 0.025, 11, 9.5))


# ---- molecular dynamics ----------------------------------------------------------------------
def test_velocity_verlet_trajectory_matches_oracle():
    s = jitter(workloads.argon_fcc(), 0.2, 4)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0))
    md.setup(s)
    md.run(s, 40)
    xo, vo, _ = orc.velocity_verlet(x0, v0, np.zeros_like(x0), 1.0, 40)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8


def test_velocity_verlet_ewald_berendsen():
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0), lg.BerendsenThermostat(250.0, 100.0))
    md.setup(s)
    md.run(s, 25)
    xo, vo, _ = orc.velocity_verlet(x0, v0, np.zeros_like(x0), 1.0, 25, 250.0, 100.0)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8


def test_berendsen_across_run_boundaries():
    """The thermostat's scaling is carried into the next step inside a run and
    applied at the end of every run: runs of 1, 3 and 21 steps give the
    oracle's 25-step trajectory."""
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    orc = oracle.Oracle(s)
    x0, v0 = s.positions.copy(), s.velocities.copy()
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0), lg.BerendsenThermostat(200.0, 10.0))
    md.setup(s)
    for k in (1, 3, 21):
        md.run(s, k)
    xo, vo, _ = orc.velocity_verlet(x0, v0, np.zeros_like(x0), 1.0, 25, 200.0, 10.0)
    assert np.abs(s.positions - xo).max() < 1e-9
    assert np.abs(s.velocities - vo).max() / np.abs(vo).max() < 1e-8


def test_md_energy_conservation_nve():
    """NVE drift bound of tests/md-nacl.rs (Ewald 5e-3 relative over the run)."""
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5, temperature=300.0)
    md = lg.MolecularDynamics(lg.VelocityVerlet(1.0))
    md.setup(s)

    def total():
        return s.potential_energy() + s.kinetic_energy()

    e0 = total()
    for _ in range(10):
        md.run(s, 50)
    assert abs((total() - e0) / e0) < 5e-3


# ---- errors mirror the reference's panics ------------------------------------------------------
def test_cutoff_above_half_cell_is_rejected():
    s = lg.System(lg.UnitCell.cubic(10.0))
    with pytest.raises(ValueError):
        s.set_pair_potential(("A", "A"), lg.PairInteraction(lg.LennardJones(1.0, 1.0), 6.0))
    eng = lg.Engine(1)
    import ctypes
    from lumol_gb300 import _capi as C
    eng.call("lg_set_cell", 0, C.dptr(np.diag([10.0, 10.0, 10.0]).ravel().copy()))
    table = (C.LgPair * 1)(C.LgPair(C.LG_PAIR_LJ, 0, 0, 0, 1.0, 1.0, 0.0, 6.0, 1.0))
    with pytest.raises(lg.EngineError):
        eng.call("lg_set_pairs", 0, 1, table)
    bad = C.LgCoulomb(C.LG_COULOMB_EWALD, 0, 0, 0, 3.0, 0.3, 1.0)
    with pytest.raises(lg.EngineError, match="kmax can not be 0"):
        eng.call("lg_set_coulomb", 0, ctypes.byref(bad))


def test_batch_of_systems_matches_each_alone():
    """Systems of one engine are independent: each one's energy, forces and
    virial equal the oracle's for that system, and computing one system leaves
    the others' device state alone."""
    from lumol_gb300.batch import Batch
    systems = [jitter(workloads.argon_fcc(cells=4), 0.2, 1), workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5),
               jitter(workloads.water_box(n_side=7, length=21.76), 0.05, 2)]
    batch = Batch(systems)
    batch.md_setup([1.0, 1.0, 0.5])
    batch.md_run(10)
    states = [batch.state(s) for s in range(3)]
    for s, system in enumerate(systems):
        system.positions = states[s][0]
        orc = oracle.Oracle(system)
        import ctypes
        from lumol_gb300 import _capi as C
        forces = np.zeros((system.size, 3))
        energy = ctypes.c_double()
        virial = np.zeros(9)
        batch.engine.call("lg_compute", s, C.dptr(np.ascontiguousarray(system.positions)), lg.LG_TERM_ALL, 7,
                          C.dptr(forces), ctypes.byref(energy), C.dptr(virial))
        assert abs(energy.value - orc.energy()) <= TOL * abs(orc.energy())
        fo = orc.forces()
        assert np.sqrt(np.mean((forces - fo) ** 2)) / np.sqrt(np.mean(fo ** 2)) <= TOL
    for s in range(3):
        pos, vel = batch.state(s)
        assert np.array_equal(pos, states[s][0]) and np.array_equal(vel, states[s][1])


# ---- cell binning of the list build --------------------------------------------------------
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_list_build_cells_match_positions(precision):
    """Every atom sits in the cell its position gives: the FP64 path bins the
    wrapped position (UnitCell::wrap_vector, cells.rs:263-270), the mixed path
    the fixed-point fraction u = floor(x 2^32 / L) mod 2^32, cell (u n) >> 32."""
    import ctypes
    import math
    from fractions import Fraction
    s = systems.random_lj_fluid(900, 0.02, 12, 9.0, family="lj", precision=precision)
    s.compute()  # builds the neighbour lists at these positions
    cells = np.zeros(s.size, dtype=np.int32)
    ncell = (ctypes.c_int32 * 3)()
    s.engine().call("lg_list_cells", 0, cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ncell)
    n = list(ncell)
    assert min(n) > 1
    expect = []
    for p in s.positions:
        c = []
        for d in range(3):
            L = s.cell.lengths[d]
            if precision == "mixed":  # (floor of the exact product)
                u = math.floor(Fraction(float(p[d])) * Fraction((1.0 / L) * 4294967296.0)) % 2 ** 32
                c.append((u * n[d]) >> 32)
            else:
                w = p[d] - math.floor(p[d] / L) * L
                c.append(min(max(int(w * (1.0 / L) * n[d]), 0), n[d] - 1))
        expect.append((c[2] * n[1] + c[1]) * n[0] + c[0])
    assert cells.tolist() == expect
