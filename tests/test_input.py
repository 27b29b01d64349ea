"""The TOML interactions reader (lumol-input/src/interactions) and the
Ewald::with_accuracy parameters it relies on.

The reference's own input tests (lumol-input/tests/input.rs:67-90) read every
file of lumol-input/tests/interactions/good without error and every case of
interactions/bad with the exact message written on its `#^ ` line; they are
run here on the reference's files where the reference tree is present.  The
other tests use inputs written here and check the values that reach the
engine."""
import glob
import os

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import refdata
import systems
from lumol_gb300 import units

INTERACTIONS = refdata.path("lumol-input", "tests", "interactions")
needs_reference = pytest.mark.skipif(not os.path.isdir(INTERACTIONS), reason=refdata.SKIP_REASON)


def _cases(kind):
    """(name, text) of every `+++`-separated case of the reference's files
    (tests/input.rs:107-150)."""
    out = []
    for path in sorted(glob.glob(os.path.join(INTERACTIONS, kind, "*.toml"))):
        text = open(path, encoding="utf-8").read()
        parts = text.split("+++")
        for i, case in enumerate(parts):
            out.append((f"{os.path.basename(path)}:{i + 1}", case))
    return out


def _message(case):
    for line in case.splitlines():
        line = line.strip()
        if line.startswith("#^ "):
            return line[3:]
    raise AssertionError("no #^ line")


def empty_system():
    """The reference reads these files into System::new(), whose cell is
    infinite: a cell large enough for every cutoff of the files stands in."""
    return lg.System(lg.UnitCell.cubic(1000.0))


@needs_reference
def test_reference_good_interaction_files():
    cases = _cases("good")
    assert len(cases) >= 8
    for name, case in cases:
        lg.InteractionsInput.from_str(case).read(empty_system())


@needs_reference
def test_reference_bad_interaction_files():
    cases = _cases("bad")
    assert len(cases) >= 80
    for name, case in cases:
        with pytest.raises(lg.InputError) as err:
            lg.InteractionsInput.from_str(case).read(empty_system())
        assert err.value.kind == "config", name
        assert err.value.reason == _message(case), name


@needs_reference
def test_reference_bench_interaction_files():
    """The interactions files of the reference's benches (benches/data/*.toml:
    argon, NaCl, water, propane) read without error."""
    files = sorted(glob.glob(refdata.path("benches", "data", "*.toml")))
    assert len(files) >= 4
    for path in files:
        s = empty_system()
        lg.InteractionsInput.new(path).read(s)
        assert s.pairs, path


def test_unit_strings():
    # units.rs tests: "10 A", kJ/mol, powers and parentheses
    assert units.from_str("10 A") == 10.0
    assert units.from_str("10") == 10.0
    assert units.from_str("5.9 kJ/mol") == units.from_(5.9, "kJ/mol")
    assert units.from_str("5 A^-1") == 5.0
    assert units.from_str("2 kJ/mol/A^2") == units.from_str("2 (kJ/mol)/(A^2)")
    assert abs(units.from_str("3 kJ^2/mol^2/A^2") / (3.0 * units.from_(1.0, "kJ/mol") ** 2) - 1.0) < 1e-15
    assert abs(units.from_str("90 deg") - np.pi / 2) < 1e-15
    for bad in ["3 foo", "3 A^", "3 (A", "x A"]:
        with pytest.raises(ValueError):
            units.from_str(bad)


PAIRS = """
[input]
version = 1

[global]
cutoff = "9 A"
tail_correction = true

[pairs]
Ar-Ar = {type = "lj", sigma = "3.405 A", epsilon = "0.996 kJ/mol"}
Ar-Kr = {type = "mie", sigma = "3.6 A", epsilon = "1.3 kJ/mol", n = 12.5, m = 6.5, cutoff = {shifted = "8.5 A"}}
Kr-Kr = {type = "lj", sigma = "3.8 A", epsilon = "1.6 kJ/mol", tail_correction = false, restriction = {scale14 = 0.5}, computation = {table = {max = "10 A", n = 4000}}}
"""


def test_pair_values_reach_the_engine():
    s = empty_system()
    lg.InteractionsInput.from_str(PAIRS).read(s)
    eps = units.from_(1.0, "kJ/mol")
    aa = lg.PairInteraction(lg.LennardJones(3.405, 0.996 * eps), 9.0)
    aa.enable_tail_corrections()
    ak = lg.PairInteraction.shifted(lg.Mie(3.6, 1.3 * eps, 12.5, 6.5), 8.5)
    ak.enable_tail_corrections()
    kk = lg.PairInteraction(lg.TableComputation(lg.LennardJones(3.8, 1.6 * eps), 4000, 10.0), 9.0)
    kk.set_restriction(lg.PairRestriction.scale14(0.5))
    for key, expected in [(("Ar", "Ar"), aa), (("Ar", "Kr"), ak), (("Kr", "Kr"), kk)]:
        got = s.pairs[key]._lower()
        want = expected._lower()
        for field, _ in got._fields_:
            assert getattr(got, field) == getattr(want, field), (key, field)


WATER = """
[input]
version = 1

[bonds]
O-H = {type = "harmonic", k = "1054.2 kcal/mol/A^2", x0 = "1.0 A"}

[angles]
H-O-H = {type = "harmonic", k = "75.9 kcal/mol/rad^2", x0 = "109.47 deg"}

[charges]
O = -0.8476
H = 0.4238

[coulomb]
ewald = {cutoff = "8.5 A", accuracy = 1e-6}
restriction = "intermolecular"
"""


def test_charges_and_ewald_accuracy():
    """ewald.rs:997-1001: Ewald::with_accuracy(8.5, 1e-6, water) has alpha
    0.2998 (to 1e-4) and kmax 5; the charges are set before the solver."""
    s = systems.ewald_water()
    for i in range(s.size):
        s.set_charge(i, 0.0)
    lg.InteractionsInput.from_str(WATER).read(s)
    assert s.charges.tolist() == [-0.8476, 0.4238, 0.4238]
    assert abs(s.coulomb.alpha - 0.2998) < 1e-4 and s.coulomb.kmax == 5
    assert s.coulomb.restriction == lg.PairRestriction.INTER_MOLECULAR
    assert s.bond_potentials[("H", "O")] == lg.Harmonic(k=units.from_(1054.2, "kcal/mol/A^2"), x0=1.0)
    assert s.angle_potentials[("H", "O", "H")].x0 == units.from_(109.47, "deg")


@pytest.mark.skipif(not refdata.available(), reason=refdata.SKIP_REASON)
def test_ewald_with_accuracy_nist_spce():
    # ewald.rs:1446-1462
    for xyz, alpha, kmax in [("spce-1.xyz", 0.2826, 5), ("spce-2.xyz", 0.2900, 5), ("spce-3.xyz", 0.2943, 5),
                             ("spce-4.xyz", 0.2912, 8)]:
        s = systems.nist_spce(refdata.path("tests", "data", "nist-spce", xyz), 9.0)
        ewald = lg.Ewald.with_accuracy(9.0, 1e-5, s)
        assert abs(ewald.alpha - alpha) < 1e-4 and ewald.kmax == kmax, xyz


def test_errors_outside_the_reference_files():
    def fails(text, message, kind="config"):
        with pytest.raises(lg.InputError) as err:
            lg.InteractionsInput.from_str(text).read(empty_system())
        assert err.value.kind == kind and err.value.reason == message

    head = "[input]\nversion = 1\n"
    fails("[pairs]\n", "missing 'input' table")
    with pytest.raises(lg.InputError) as err:
        lg.InteractionsInput.from_str("[input]\nversion = \n")
    assert err.value.kind == "toml"
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", restriction = "scale14"}',
          "'scale14' restriction must be a table")
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", restriction = "bonded"}',
          "Unknown restriction 'bonded'")
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", restriction = {scale14 = 1}}',
          "'scale14' parameter must be a float")
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", restriction = {scale13 = 0.5}}',
          "Restriction table must be 'scale14'")
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", computation = {spline = {}}}',
          "Unknown computation type 'spline'")
    fails(head + '[pairs]\nA-A = {type = "null", cutoff = "3 A", computation = {table = {max = "3 A"}}}',
          "missing 'n' key in table computation")
    fails(head + '[global]\ntail_correction = 1\n[pairs]\nA-A = {type = "null", cutoff = "3 A"}',
          "the 'tail_correction' section must be a boolean value")
    fails(head + '[bonds]\nA-A = {type = "torsion", k = "1 kJ/mol", delta = "1 deg", n = 2}',
          "unknown potential type 'torsion'")
    fails(head + "[coulomb]\nrestriction = \"none\"\n", "got more than one coulombic solver: ")


MORSE_CHAINS = """
[input]
version = 1

[global]
cutoff = "7 A"

[pairs]
C-C = {type = "lj", sigma = "3.4 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}
C-O = {type = "lj", sigma = "3.2 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}
C-N = {type = "lj", sigma = "3.3 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}
O-O = {type = "lj", sigma = "3.0 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}
O-N = {type = "lj", sigma = "3.1 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}
N-N = {type = "lj", sigma = "3.25 A", epsilon = "0.5 kJ/mol", restriction = "exclude13"}

[bonds]
C-C = {type = "morse", A = "2.1 A^-1", depth = "350 kJ/mol", x0 = "1.2 A"}
C-O = {type = "harmonic", k = "2500 kJ/mol/A^2", x0 = "1.3 A"}
C-N = {type = "morse", A = "1.9 A^-1", depth = "300 kJ/mol", x0 = "1.25 A"}

[angles]
C-C-O = {type = "morse", A = "2.5 rad^-1", depth = "120 kJ/mol", x0 = "109 deg"}
C-O-C = {type = "harmonic", k = "320 kJ/mol/rad^2", x0 = "1.95 rad"}
O-C-N = {type = "cosine-harmonic", k = "250 kJ/mol", x0 = "2.0 rad"}

[dihedrals]
C-C-O-C = {type = "torsion", n = 3, k = "5 kJ/mol", delta = "0.4 rad"}
C-O-C-N = {type = "morse", A = "1.5 rad^-1", depth = "8 kJ/mol", x0 = "100 deg"}

[coulomb]
wolf = {cutoff = "8 A"}
restriction = "exclude13"
"""


def test_morse_bonded_oracle_matches_reference_formula():
    """Morse as bond / angle / dihedral potential (functions.rs:414-437):
    the oracle's energy and force at a few points, against the formula."""
    a, x0, depth = 2.0, 1.3, 4.0
    for x in (0.7, 1.0, 1.3, 2.2):
        e, f = oracle.bonded_eval(oracle.MORSE, depth, x0, x, a=a)
        ex = np.exp((x0 - x) * a)
        assert e == depth * (1.0 - ex) * (1.0 - ex)
        assert f == 2.0 * depth * (1.0 - ex * ex) * a
    # the reference's doc test (functions.rs:400-402)
    e, f = oracle.bonded_eval(oracle.MORSE, 4.0, 1.3, 1.0, a=2.0)
    assert e == 2.703517287822119 and f == -37.12187076378477


@pytest.mark.gpu
def test_interactions_from_toml_match_oracle():
    """Chains whose interactions come from a TOML file, with Morse bonds,
    angles and dihedral angles: energies, forces and virial against the
    oracle."""
    from test_gpu_parity import assert_parity
    s = systems.chains(27, 24.0, 9, lg.PairRestriction.NONE)
    s.pairs.clear()
    s.bond_potentials.clear()
    s.angle_potentials.clear()
    lg.InteractionsInput.from_str(MORSE_CHAINS).read(s)
    assert isinstance(s.bond_potentials[("C", "C")], lg.Morse)
    assert isinstance(s.dihedral_potential(("N", "C", "O", "C")), lg.Morse)
    assert_parity(s)


def test_rotation_matrix_literal():
    """types/matrix.rs:136-148: a quarter turn around 2 e1 takes e3 to e2."""
    from lumol_gb300.system import _rotation
    r = _rotation(np.array([2.0, 0.0, 0.0]), np.radians(90.0))
    assert np.array_equal(np.round(r @ [0.0, 0.0, 1.0] * 1e8) / 1e8, [0.0, 1.0, 0.0])
    assert np.allclose(r @ r.T, np.eye(3), atol=1e-15)
