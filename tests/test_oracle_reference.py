"""Pins the CPU oracle to the reference: its unit-test literals and the NIST
LJ / SPC/E known answers (read from the reference tree at test time).

Each test names the reference test it restates.  Tolerances are the
reference's own (assert_eq / assert_ulps_eq / relative bounds)."""
import math

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import refdata
import systems
from lumol_gb300 import units
from ulps import relative_eq, rust_round_at, ulps_eq

LJ, BUCK, HARM, BMH, MORSE, GAUSS, MIE = 2, 3, 4, 5, 6, 7, 8
needs_reference = pytest.mark.skipif(not refdata.available(), reason=refdata.SKIP_REASON)


# ---- energy/functions.rs:621-715 ---------------------------------------------
def test_lennard_jones_literals(oracle_lib):
    e = lambda r: oracle.pair_eval(LJ, (2.0, 0.8), 1e9, r)
    assert e(2.0)[0] == 0.0
    assert e(2.5)[0] == -0.6189584744448002
    tail = lambda rc: oracle.pair_eval(LJ, (2.0, 0.8), rc, 1.0, tail=True)
    assert tail(1.0)[2] == 1388.0888888888887
    assert tail(2.0)[2] == -5.688888888888889
    assert tail(14.42)[2] == -0.022767318648783084
    assert tail(1.0)[3] == 17066.666666666668
    assert tail(2.0)[3] == -17.06666666666667
    assert tail(14.42)[3] == -0.1366035877536718
    assert abs(e(2.0 ** (1.0 / 6.0) * 2.0)[1]) < 1e-15
    assert ulps_eq(e(2.5)[1], -0.95773475733504)
    eps = 1e-9
    assert relative_eq((e(4.0)[0] - e(4.0 + eps)[0]) / eps, e(4.0)[1], epsilon=1e-6)


def test_harmonic_literals(oracle_lib):
    h = lambda r: oracle.pair_eval(HARM, (50.0, 2.0), 1e9, r)
    assert h(2.0)[0] == 0.0
    assert h(2.5)[0] == 6.25
    assert h(2.0)[1] == 0.0
    assert h(2.5)[1] == -25.0


def test_buckingham_literals(oracle_lib):
    b = lambda r: oracle.pair_eval(BUCK, (2.0, 1.0, 2.0), 1e9, r)
    assert b(2.0)[0] == 0.7201338823428847
    assert b(2.0)[1] == 0.32100444117144233
    t = oracle.pair_eval(BUCK, (2.0, 1.0, 2.0), 10.0, 1.0, tail=True)
    assert t[2] == 1.8323882504179136
    assert t[3] == 33.422487868546725  # includes the reference's "+ 8.0" (functions.rs:317)
    # doc test of functions.rs:271-274
    d = lambda r: oracle.pair_eval(BUCK, (2.0, 1.0, 5.3), 1e9, r)
    assert d(2.2)[0] == 1.3117360696239022
    assert d(2.2)[1] == 0.2251072178835946


def test_born_mayer_huggins_literals(oracle_lib):
    # functions.rs:718-737: BornMayerHuggins {a, c, d, sigma, rho}
    b = lambda r: oracle.pair_eval(BMH, (2.0, 1.0, 0.5, 2.0, 2.0), 1e9, r)
    assert b(2.0)[0] == 1.986328125
    assert b(2.0)[1] == 0.9609375
    t = oracle.pair_eval(BMH, (2.0, 1.0, 0.5, 2.0, 2.0), 10.0, 1.0, tail=True)
    assert t[2] == 4.981521444402363
    assert t[3] == 69.13986044386026
    eps = 1e-9
    assert relative_eq((b(4.0)[0] - b(4.0 + eps)[0]) / eps, b(4.0)[1], epsilon=1e-6)
    # doc test of functions.rs:335-337
    d = lambda r: oracle.pair_eval(BMH, (2.0, 1.0, 0.5, 1.5, 5.3), 1e9, r)
    assert d(2.2)[0] == 1.7446409593340713
    assert d(2.2)[1] == 0.30992873382584607


def test_morse_literals(oracle_lib):
    # functions.rs:739-757 and the doc test of functions.rs:400-402: Morse {a, x0, depth}
    m = lambda r: oracle.pair_eval(MORSE, (2.0, 1.3, 4.0), 1e9, r)
    assert m(1.0)[0] == 2.703517287822119
    assert m(1.0)[1] == -37.12187076378477
    t = oracle.pair_eval(MORSE, (2.0, 1.3, 4.0), 1.0, 1.0, tail=True)
    assert t[2] == 0.0 and t[3] == 0.0
    # the reference's force is 2·depth·(1 - e²)·a, not the derivative of its
    # energy; its finite-difference check passes at r = x0 where both vanish
    eps = 1e-9
    assert relative_eq((m(1.3)[0] - m(1.3 + eps)[0]) / eps, m(1.3)[1], epsilon=1e-6)


def test_gaussian_literals(oracle_lib):
    # functions.rs:759-772: Gaussian::new(a, b)
    g = lambda r: oracle.pair_eval(GAUSS, (8.0, 2.0), 1e9, r)
    assert g(0.0)[0] == -8.0
    assert g(0.0)[1] == 0.0
    t = oracle.pair_eval(GAUSS, (8.0, 2.0), 2.5, 1.0, tail=True)
    assert relative_eq(t[2], -1.93518e-5, epsilon=1e-10)
    assert relative_eq(t[3], 5.23887e-4, epsilon=1e-10)
    eps = 1e-9
    assert relative_eq((g(0.5)[0] - g(0.5 + eps)[0]) / eps, g(0.5)[1], epsilon=1e-6)
    # doc test of functions.rs:454-456
    assert oracle.pair_eval(GAUSS, (8.0, 0.5), 1e9, 0.0)[:2] == (-8.0, 0.0)


def test_mie_literals(oracle_lib):
    # functions.rs:780-801: Mie::new(sigma, epsilon, n, m)
    m = lambda r: oracle.pair_eval(MIE, (2.0, 0.8, 12.0, 6.0), 1e9, r)
    assert m(2.0)[0] == 0.0
    assert m(2.5)[0] == -0.6189584744448002
    tail = lambda rc: oracle.pair_eval(MIE, (2.0, 0.8, 12.0, 6.0), rc, 1.0, tail=True)
    assert relative_eq(tail(1.0)[2], 1388.0888889, epsilon=1e-6)
    assert relative_eq(tail(2.0)[2], -5.688888888888889, epsilon=1e-6)
    assert relative_eq(tail(14.42)[2], -0.022767318648783084, epsilon=1e-6)
    assert relative_eq(tail(1.0)[3], 17066.666666666668, epsilon=1e-6)
    assert relative_eq(tail(2.0)[3], -17.06666666666667, epsilon=1e-6)
    assert relative_eq(tail(14.42)[3], -0.1366035877536718, epsilon=1e-6)
    assert abs(m(2.0 ** (1.0 / 6.0) * 2.0)[1]) < 1e-15
    assert ulps_eq(m(2.5)[1], -0.95773475733504)
    eps = 1e-9
    assert relative_eq((m(4.0)[0] - m(4.0 + eps)[0]) / eps, m(4.0)[1], epsilon=1e-6)
    # functions.rs:809-815: no tail correction when m <= 3
    t = oracle.pair_eval(MIE, (2.0, 0.8, 12.0, 2.0), 2.0, 1.0, tail=True)
    assert t[2] == 0.0 and t[3] == 0.0
    # doc test of functions.rs:520-524
    d = lambda r: oracle.pair_eval(MIE, (2.0, 10.0, 12.0, 6.0), 1e9, r)
    assert d(2.0)[0] == 0.0
    assert abs(d(3.0)[0] + 3.203365942785746) < 1e-8
    assert d(2.0)[1] == 120.0


def test_table_computation_literals(oracle_lib):
    # computations.rs:180-205: TableComputation of Harmonic {k 50, x0 2}, 1000 points up to 4
    t = lambda r: oracle.pair_eval(HARM, (50.0, 2.0), 1e9, r, table=(1000, 4.0))
    assert t(2.5)[:2] == (6.25, -25.0)
    delta = 4.0 / 1000.0
    assert t(4.0 - 2.0 * delta)[:2] == (99.2016, -99.6)
    for r in (4.0 - delta, 4.0, 4.1):
        assert t(r)[:2] == (0.0, 0.0)
    # the tail corrections are the potential's own
    lj = oracle.pair_eval(LJ, (2.0, 50.0), 5.0, 1.0, tail=True)
    tab = oracle.pair_eval(LJ, (2.0, 50.0), 5.0, 1.0, tail=True, table=(1000, 4.0))
    assert tab[2:] == lj[2:]
    # doc test of computations.rs:92-100: Harmonic {x0 0.5, k 4.2}, 1000 points up to 2
    d = lambda r: oracle.pair_eval(HARM, (4.2, 0.5), 1e9, r, table=(1000, 2.0))
    assert d(1.0)[0] == 0.525
    assert d(3.0)[0] == 0.0


def test_cosine_harmonic_and_torsion_literals(oracle_lib):
    # functions.rs:663-697 and the doc tests of functions.rs:173-177, 228-232
    cos = lambda x: oracle.bonded_eval(oracle.COSINE_HARMONIC, 50.0, 2.0, x)
    assert cos(2.0) == (0.0, 0.0)
    dcos = math.cos(2.5) - math.cos(2.0)
    assert cos(2.5) == (0.5 * 50.0 * dcos * dcos, 50.0 * dcos * math.sin(2.5))
    eps = 1e-9
    assert relative_eq((cos(2.3)[0] - cos(2.3 + eps)[0]) / eps, cos(2.3)[1], epsilon=1e-6)
    assert oracle.bonded_eval(oracle.COSINE_HARMONIC, 100.0, 2.0, 3.0)[0] == 16.464942078100552
    tor = lambda x: oracle.bonded_eval(oracle.TORSION, 5.0, 3.0, x, n=3)
    assert tor(1.0) == (10.0, 0.0)
    assert tor(1.1)[0] == 5.0 * (1.0 + math.cos(3.0 * 1.1 - 3.0))
    assert relative_eq((tor(4.0)[0] - tor(4.0 + eps)[0]) / eps, tor(4.0)[1], epsilon=1e-6)
    doc = lambda x: oracle.bonded_eval(oracle.TORSION, 10.0, math.pi / 2.0, x, n=3)
    assert doc(math.pi / 2.0)[0] == 0.0
    assert doc(math.pi / 3.0)[0] == 10.0
    assert abs(doc(math.pi / 2.0)[1]) < 1e-12


def test_dihedral_geometry_literals(oracle_lib):
    # sys/config/cells.rs:746-797
    phi, _ = oracle.dihedral_geometry([0, 0, 0], [1, 0, 0], [1, 1, 0], [2, 1, 0])
    assert phi == math.pi
    pts = [np.array(p) for p in ([1.241, 0.444, 0.349], [-0.011, -0.441, 0.333], [-1.176, 0.296, -0.332],
                                 [-1.396, 1.211, 0.219])]
    phi, d = oracle.dihedral_geometry(*pts)
    assert relative_eq(phi, -1.0453789626063168)
    eps = 1e-6
    for a in range(4):
        for k in range(3):
            moved = [p.copy() for p in pts]
            moved[a][k] += eps
            fd = (oracle.dihedral_geometry(*moved)[0] - phi) / eps
            assert ulps_eq(fd, d[a][k], epsilon=1e-6)


def test_dihedrals_of_the_host_match_the_oracle(oracle_lib):
    s = systems.chains(8, 30.0, 3, lg.PairRestriction.INTER_MOLECULAR, dihedrals=True)
    orc = oracle.Oracle(s)
    assert orc.dihedrals().tolist() == [list(d) for d in s.dihedrals()]
    assert len(s.dihedrals()) == 16


# ---- energy/pairs.rs:317-360 ----------------------------------------------------
def test_pair_interaction_literals(oracle_lib):
    cut = lambda r: oracle.pair_eval(LJ, (1.0, 2.0), 4.0, r)
    lj = lambda r: oracle.pair_eval(LJ, (1.0, 2.0), 1e9, r)
    assert cut(2.5)[:2] == lj(2.5)[:2]
    assert cut(4.1)[:2] == (0.0, 0.0)
    shifted = lambda r: oracle.pair_eval(LJ, (1.0, 2.0), 4.0, r, shifted=True, tail=True)
    assert ulps_eq(shifted(2.5)[1], lj(2.5)[1])
    assert ulps_eq(shifted(2.5)[0], -0.030681134109158216)
    assert shifted(4.1)[:2] == (0.0, 0.0)
    assert shifted(1.0)[2] == -0.041663275824652776
    # tail_virial() is tail_virial(rc) * one / 3; its trace adds the three diagonal entries
    w = shifted(1.0)[3] * (1.0 / 3.0)
    assert ulps_eq(w + w + w, -0.24995930989583334)
    # doc tests of pairs.rs:254-296
    assert oracle.pair_eval(LJ, (0.5, 4.2), 2.0, 1.0, tail=True)[2] == -0.010936609903971353
    assert oracle.pair_eval(LJ, (0.5, 4.2), 2.0, 1.0, tail=True)[3] * (1.0 / 3.0) == -0.02187143961588542
    assert oracle.pair_eval(HARM, (4.2, 0.5), 2.0, 1.0)[0] == 0.525
    assert oracle.pair_eval(HARM, (4.2, 0.5), 2.0, 2.0)[0] == 0.0
    assert oracle.pair_eval(HARM, (4.2, 0.5), 2.0, 1.0, shifted=True)[0] == -4.2


# ---- sys/energy.rs:224-263 --------------------------------------------------------
def test_energy_evaluator_literals(oracle_lib):
    orc = oracle.Oracle(systems.evaluator_system())
    assert ulps_eq(orc.energy(oracle.TERM_PAIRS), units.from_(-258.3019360389957, "kJ/mol"))
    assert ulps_eq(orc.energy(oracle.TERM_TAIL), -0.0000028110338032153973)
    assert ulps_eq(orc.energy(oracle.TERM_BONDS), units.from_(150.0, "kJ/mol"))
    assert ulps_eq(orc.energy(oracle.TERM_ANGLES), units.from_(400.0, "kJ/mol"))


def test_bonding_angles_match_host_derivation(oracle_lib):
    s = systems.chains(3, 30.0, 0, 0)
    orc = oracle.Oracle(s)
    assert orc.angles().tolist() == [list(a) for a in s.angles()]


# ---- energy/global/ewald.rs:1041-1193 -----------------------------------------------
def test_ewald_nacl_pair(oracle_lib):
    import lumol_gb300 as lg
    s = systems.nacl_pair()
    s.set_coulomb_potential(lg.Ewald(8.0, 10))
    orc = oracle.Oracle(s)
    e = orc.energy()
    assert ulps_eq(e, -0.09262397663346732, epsilon=1e-4)
    f = orc.forces()
    assert ulps_eq(float(np.linalg.norm(f[0] + f[1])), 0.0)
    assert f[0, 0] > 0.0 and f[1, 0] < 0.0
    # finite differences (ewald.rs:1057-1114)
    eps = 1e-9
    for terms in (oracle.TERM_COUL_REAL, oracle.TERM_ALL):
        e0 = orc.energy(terms)
        pos = s.positions.copy()
        pos[0, 0] += eps
        orc.set_positions(pos)
        e1 = orc.energy(terms)
        orc.set_positions(s.positions)
        assert relative_eq((e0 - e1) / eps, orc.forces(terms)[0, 0], epsilon=1e-6)
    s2 = systems.nacl_pair()
    s2.set_coulomb_potential(lg.Ewald(2.0, 10))
    orc2 = oracle.Oracle(s2)
    e0 = orc2.energy(oracle.TERM_COUL_KSPACE)
    pos = s2.positions.copy()
    pos[0, 0] += eps
    orc2.set_positions(pos)
    e1 = orc2.energy(oracle.TERM_COUL_KSPACE)
    orc2.set_positions(s2.positions)
    assert relative_eq((e0 - e1) / eps, orc2.forces(oracle.TERM_COUL_KSPACE)[0, 0], epsilon=1e-6)


def test_ewald_water_energy(oracle_lib):
    import lumol_gb300 as lg
    s = systems.ewald_water()
    ew = lg.Ewald(8.0, 10)
    ew.set_restriction(lg.PairRestriction.INTER_MOLECULAR)
    s.set_coulomb_potential(ew)
    orc = oracle.Oracle(s)
    # ewald.rs:1124-1134 (assert_ulps_eq): erfc comes from libm here, from `special` there
    assert ulps_eq(orc.energy(), -0.000009243868813825495, max_ulps=4, epsilon=1e-16)


def test_ewald_virial_is_energy(oracle_lib):
    # ewald.rs:1216-1231: for point charges the Ewald energy equals the virial trace
    import lumol_gb300 as lg
    for make in (systems.ewald_water, systems.nacl_pair):
        s = make()
        s.set_coulomb_potential(lg.Ewald(8.0, 10))
        orc = oracle.Oracle(s)
        e = orc.energy()
        w = float(np.trace(orc.virial()))
        assert relative_eq(e, w, max_relative=1e-3)


@pytest.mark.parametrize("terms,cutoff", [(oracle.TERM_COUL_REAL, 8.0), (oracle.TERM_COUL_KSPACE, 2.0)])
def test_ewald_virial_finite_differences(oracle_lib, terms, cutoff):
    # ewald.rs:1233-1284, diagonal entries (orthorhombic cells only)
    import lumol_gb300 as lg

    def build(scale):
        s = systems.ewald_water()
        s.cell = lg.UnitCell.ortho(*[20.0 * f for f in scale])
        s.positions = s.positions * np.array(scale)
        ew = lg.Ewald(cutoff, 10)
        ew.set_restriction(lg.PairRestriction.INTER_MOLECULAR)
        s.coulomb = ew
        return oracle.Oracle(s)

    virial = build([1.0, 1.0, 1.0]).virial(terms)
    eps = 1e-9
    for i in range(3):
        scale = [1.0, 1.0, 1.0]
        scale[i] += eps
        fd = (build([1.0, 1.0, 1.0]).energy(terms) - build(scale).energy(terms)) / eps
        assert relative_eq(virial[i, i], fd, epsilon=1e-6)


# ---- energy/global/wolf.rs tests ---------------------------------------------------------
def test_wolf_nacl_pair(oracle_lib):
    import lumol_gb300 as lg
    s = systems.nacl_pair()
    s.set_coulomb_potential(lg.Wolf(8.0))
    orc = oracle.Oracle(s)
    assert ulps_eq(orc.energy(), -0.09262397663346732, epsilon=1e-2)
    f = orc.forces()
    assert ulps_eq(float(np.linalg.norm(f[0] + f[1])), 0.0)
    eps = 1e-9
    e0 = orc.energy()
    pos = s.positions.copy()
    pos[0, 0] += eps
    orc.set_positions(pos)
    e1 = orc.energy()
    orc.set_positions(s.positions)
    assert relative_eq((e0 - e1) / eps, f[0, 0], epsilon=1e-6)


# ---- sys/cache.rs:295-485 and ewald.rs:1288-1377: move cost equals the energy change --------
@pytest.mark.parametrize("coulomb", ["none", "ewald", "wolf"])
def test_cache_cost_is_energy_difference(oracle_lib, coulomb):
    import lumol_gb300 as lg
    s = systems.chains(8, 22.0, 3, lg.PairRestriction.INTER_MOLECULAR,
                       coulomb={"none": None, "ewald": lg.Ewald(9.0, 5, 0.35), "wolf": lg.Wolf(9.0)}[coulomb])
    orc = oracle.Oracle(s)
    orc.cache_init()
    e_before = orc.energy()
    assert relative_eq(orc.cache_energy(), e_before, epsilon=1e-12 * abs(e_before))
    lo, hi = s.molecule_range(3)
    newpos = s.positions[lo:hi] + np.array([0.4, -0.3, 0.25])
    cost = orc.move_molecule_cost(3, newpos)
    pos = s.positions.copy()
    pos[lo:hi] = newpos
    orc.set_positions(pos)
    e_after = orc.energy()
    assert abs(cost - (e_after - e_before)) <= 1e-9 * max(1.0, abs(e_before))
    orc.cache_update()
    assert abs(orc.cache_energy() - e_after) <= 1e-9 * max(1.0, abs(e_after))


# ---- sys/cache.rs:450-484 (move_all_molecules) and a Resize-like cell change --------------
@pytest.mark.parametrize("coulomb", ["none", "ewald", "wolf"])
def test_cache_all_molecules_cost_is_energy_difference(oracle_lib, coulomb):
    """cost == E(new) - E(old) (cache.rs:450-484, epsilon 1e-12 there) for a
    rigid translation of every molecule, then for a Resize of the cell with
    the centres of mass scaled (resize.rs:70-107); the update keeps the new
    configuration, the restore puts the old one back."""
    import lumol_gb300 as lg
    mk = lambda: systems.chains(8, 22.0, 3, lg.PairRestriction.INTER_MOLECULAR,
                                coulomb={"none": None, "ewald": lg.Ewald(9.0, 5, 0.35),
                                         "wolf": lg.Wolf(9.0)}[coulomb])
    s = mk()
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = orc.energy()
    L = np.array(s.cell.lengths)
    pos1 = s.positions + np.array([-0.9, 0.0, 1.8])
    cost = orc.move_all_molecules_cost(L, pos1)
    ref = oracle.Oracle(mk())
    ref.set_positions(pos1)
    e1 = ref.energy()
    assert abs(cost - (e1 - e0)) <= 1e-10 * max(1.0, abs(e0))
    orc.cache_update()
    assert abs(orc.cache_energy() - e1) <= 1e-10 * max(1.0, abs(e1))
    # a Resize: cell x 1.02, each molecule moved with its centre of mass
    L2 = L * 1.02
    m = s.masses
    pos2 = pos1.copy()
    for mol in range(int(s.molecules.max()) + 1):
        lo, hi = s.molecule_range(mol)
        com = (m[lo:hi, None] * pos1[lo:hi]).sum(axis=0) / m[lo:hi].sum()
        pos2[lo:hi] += com / L * L2 - com
    cost2 = orc.move_all_molecules_cost(L2, pos2)
    ref2 = oracle.Oracle(mk())
    ref2.set_cell(L2)
    ref2.set_positions(pos2)
    e2 = ref2.energy()
    assert abs(cost2 - (e2 - e1)) <= 1e-10 * max(1.0, abs(e0))
    orc.cache_restore()  # rejected: back to the translated configuration
    assert np.allclose(orc.cell(), L, rtol=0, atol=0)
    assert abs(orc.energy() - e1) <= 1e-12 * max(1.0, abs(e1))


# ---- tests/nist-lj.rs ----------------------------------------------------------------------
@needs_reference
@pytest.mark.parametrize("case", range(8))
def test_nist_lj(oracle_lib, case):
    cutoff, xyz, checks = refdata.nist_lj_cases()[case]
    orc = oracle.Oracle(systems.nist_lj(xyz, cutoff, tail=False))
    energy = orc.energy()
    virial = float(np.trace(orc.virial()))
    tail = oracle.Oracle(systems.nist_lj(xyz, cutoff, tail=True)).energy() - energy
    values = {"energy": energy, "virial": virial, "tail": tail}
    for what, dec, expected in checks:
        assert rust_round_at(values[what], dec) == expected, (what, values[what], expected)


# ---- tests/nist-spce.rs --------------------------------------------------------------------
@needs_reference
@pytest.mark.parametrize("case", range(8))
def test_nist_spce_energies(oracle_lib, case):
    cutoff, xyz, checks = refdata.nist_spce_cases()[case]
    orc = oracle.Oracle(systems.nist_spce(xyz, cutoff))
    kb = units.K_BOLTZMANN
    values = {
        "total": orc.energy() / kb,
        "pairs": orc.energy(oracle.TERM_PAIRS) / kb,
        "tail": orc.energy(oracle.TERM_TAIL) / kb,
        "coulomb": orc.energy(oracle.TERM_COUL_REAL | oracle.TERM_COUL_SELF | oracle.TERM_COUL_KSPACE) / kb,
    }
    for what, expected in checks:
        assert abs((values[what] - expected) / expected) < 1e-3, (what, values[what], expected)


@needs_reference
@pytest.mark.parametrize("case", [0, 1, 4, 5])
def test_nist_spce_forces_against_lammps(oracle_lib, case):
    cutoff, kmax, alpha, xyz, ffile, dynamic = refdata.nist_spce_force_cases()[case]
    orc = oracle.Oracle(systems.nist_spce(xyz, cutoff, lammps=(kmax, alpha)))
    forces = np.array([[units.to(x, "kcal/mol/A") for x in f] for f in orc.forces()])
    expected = refdata.read_forces(ffile)
    rel = np.abs((forces - expected) / expected)
    if dynamic:
        tol = np.where(np.abs(expected) < 1e-1, 1e-1, np.where(np.abs(expected) < 1.0, 5e-2, 1e-2))
    else:
        tol = 5e-3
    assert np.all(rel < tol), float(rel.max())
