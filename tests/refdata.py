"""Known-answer data of the reference, read from its source tree at test time.

The NIST LJ / SPC/E reference values live in the reference's own integration
tests (tests/nist-lj.rs, tests/nist-spce.rs) together with the configurations
they apply to (tests/data/nist-*).  Nothing is copied into this repository:
these helpers parse the assertions and the data files where they lie, and the
tests that use them are skipped when the reference tree is not present.

The reference tree is the directory named by the environment variable
LUMOL_REFERENCE_ROOT; without it, a checkout named `reference` beside this
repository's root directory is used when one exists.
"""
from __future__ import annotations

import os
import re

import numpy as np

_REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE_ROOT = os.environ.get("LUMOL_REFERENCE_ROOT") or os.path.join(os.path.dirname(_REPO), "reference")
SKIP_REASON = ("reference tree not found: set LUMOL_REFERENCE_ROOT to a lumol checkout "
               "(or place one beside this repository as `reference`)")


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "tests", "data"))


def path(*parts: str) -> str:
    return os.path.join(REFERENCE_ROOT, *parts)


def read_xyz(file: str):
    """(names, positions, cell lengths) of an XYZ file whose comment line
    holds `cell: a [b c]`."""
    with open(file) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    cell = [float(x) for x in lines[1].split(":")[1].split()]
    if len(cell) == 1:
        cell = cell * 3
    names, pos = [], []
    for line in lines[2 : 2 + n]:
        parts = line.split()
        names.append(parts[0])
        pos.append([float(x) for x in parts[1:4]])
    return names, np.array(pos), tuple(cell)


def read_forces(file: str) -> np.ndarray:
    """LAMMPS forces file of tests/data/nist-spce (index fx fy fz, kcal/mol/A)."""
    with open(file) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    out = np.zeros((n, 3))
    for i, line in enumerate(lines[2 : 2 + n]):
        parts = line.split()
        assert int(parts[0]) == i + 1
        out[i] = [float(x) for x in parts[1:4]]
    return out


def nist_lj_cases():
    """[(cutoff, data file, [(quantity, decimals, value)])] from tests/nist-lj.rs."""
    src = open(path("tests", "nist-lj.rs")).read()
    cases = []
    for mod in re.split(r"\nmod ", src)[1:]:
        cut = re.search(r"PairInteraction::new\(\s*Box::new\(LennardJones\s*\{[^}]*\}\),\s*([0-9.]+),", mod, re.S)
        cutoff = float(cut.group(1))
        for fn in re.split(r"fn nist\d+\(\)", mod)[1:]:
            toml = re.search(r'let path = "(lj-\d+)\.toml"', fn).group(1)
            checks = []
            for what, dec, val in re.findall(r"assert_eq!\((energy|virial|tail)\.round_at\((\d+)\),\s*([-0-9.]+)\)", fn):
                checks.append((what, int(dec), float(val)))
            cases.append((cutoff, path("tests", "data", "nist-lj", toml + ".xyz"), checks))
    return cases


def nist_spce_cases():
    """Energy checks of tests/nist-spce.rs:
    [(cutoff, xyz file, [(quantity, expected / K_BOLTZMANN)])]."""
    src = open(path("tests", "nist-spce.rs")).read()
    cases = []
    for fn in re.findall(r"fn nist\d\(\)\s*\{(.*?)\n    \}", src, re.S):
        xyz = re.search(r'get_system\("(spce-\d\.xyz)"\)', fn).group(1)
        cutoff = float(re.search(r"set_nist_interactions\(&mut system, ([0-9.]+)\)", fn).group(1))
        checks = re.findall(
            r"let energy = (system\.potential_energy\(\)|evaluator\.pairs\(\)|evaluator\.pairs_tail\(\)|"
            r"evaluator\.coulomb\(\)) / K_BOLTZMANN;\s*let expected = ([-0-9.e]+);", fn)
        names = {"system.potential_energy()": "total", "evaluator.pairs()": "pairs",
                 "evaluator.pairs_tail()": "tail", "evaluator.coulomb()": "coulomb"}
        cases.append((cutoff, path("tests", "data", "nist-spce", xyz),
                       [(names[w], float(v)) for w, v in checks]))
    return cases


def nist_spce_force_cases():
    """[(cutoff, kmax, alpha, xyz file, forces file, dynamic tolerance?)] of tests/nist-spce.rs."""
    src = open(path("tests", "nist-spce.rs")).read()
    out = []
    for mod in re.split(r"\nmod ", src)[1:]:
        for fn in re.findall(r"fn nist\d_forces\(\)\s*\{(.*?)\n    \}", mod, re.S):
            xyz = re.search(r'get_system\("(spce-\d\.xyz)"\)', fn).group(1)
            cut, kmax, alpha = re.search(
                r"set_lammps_interactions\(&mut system, ([0-9.]+), (\d+), ([0-9.]+)\)", fn).groups()
            forces = re.search(r'get_forces\("(forces-[0-9-]+\.xyz)"\)', fn).group(1)
            dynamic = "Dynamic tolerance" in fn
            out.append((float(cut), int(kmax), float(alpha), path("tests", "data", "nist-spce", xyz),
                        path("tests", "data", "nist-spce", forces), dynamic))
    return out
