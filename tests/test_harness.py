"""The C++ replay harness (tests/harness/replay.cpp): Lumol's host call
sequence (Forces / PotentialEnergy / AtomicVirial of sys/compute.rs, the
VelocityVerlet steps of md/integrators.rs, the cutoff check of
sys/system.rs:122-131) through the C ABI with no Python in between.

CPU: the harness compiles and links against include/lumol_gb300.h and the
engine library, and without a GPU it fails loudly (exit 3, no CPU fallback).
GPU: its own checks pass, and its energy, virial and 10-step trajectory equal
the oracle's for the same NaCl crystal (1e-10, 1e-9 A)."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available

SRC = os.path.join(ROOT, "tests", "harness", "replay.cpp")


def build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from lumol_gb300 import _capi
    libdir = os.path.dirname(_capi.LIB_PATH)
    exe = str(tmp_path / "replay")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-o", exe, SRC, f"-L{libdir}", "-llumol_gb300",
           f"-Wl,-rpath,{libdir}"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return exe


def write_input(path, system, cutoff, alpha, kmax):
    # the LJ parameters of the NaCl workload (workloads.nacl_crystal) in internal units
    from lumol_gb300.units import from_
    eps = (from_(0.544, "kJ/mol"), from_(0.4184, "kJ/mol"))
    with open(path, "w") as f:
        f.write(f"{system.size} {float(system.cell.lengths[0])!r} {float(cutoff)!r} {float(alpha)!r} {kmax}\n")
        f.write(f"{2.35!r} {4.40!r} {float(eps[0])!r} {float(eps[1])!r}\n")
        for k, q, m, x in zip(system.kinds, system.charges, system.masses, system.positions):
            vals = " ".join(repr(float(v)) for v in (q, m, x[0], x[1], x[2]))
            f.write(f"{int(k)} {vals}\n")


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_harness_builds_and_fails_loudly_without_a_gpu(tmp_path):
    from lumol_gb300 import workloads
    exe = build(tmp_path)
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    write_input(tmp_path / "in.txt", s, 8.0, 0.35, 5)
    out = subprocess.run([exe, str(tmp_path / "in.txt")], capture_output=True, text=True)
    assert out.returncode == 3, (out.returncode, out.stdout, out.stderr)
    assert "no CPU fallback" in out.stdout


@pytest.mark.gpu
def test_harness_replays_lumols_call_sequence(tmp_path):
    import oracle
    from lumol_gb300 import workloads
    exe = build(tmp_path)
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    write_input(tmp_path / "in.txt", s, 8.0, 0.35, 5)
    out = subprocess.run([exe, str(tmp_path / "in.txt")], capture_output=True, text=True)
    assert out.returncode == 0, (out.stdout, out.stderr)
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["failures"] == 0
    from lumol_gb300 import _capi as C
    orc = oracle.Oracle(s)
    e, w = orc.energy(), orc.virial().ravel()
    assert abs(res["energy"] - e) <= 1e-10 * abs(e)
    # the total virial of the crystal is a small difference of the pair and
    # Coulomb virials: the tolerance is relative to the larger of the two
    groups = (C.LG_TERM_PAIRS | C.LG_TERM_TAIL, C.LG_TERM_COUL_REAL | C.LG_TERM_COUL_SELF | C.LG_TERM_COUL_KSPACE)
    scale = max(np.abs(orc.virial(t)).max() for t in groups)
    assert np.abs(np.array(res["virial"]) - w).max() <= 1e-10 * scale
    x, v, _ = orc.velocity_verlet(s.positions, np.zeros_like(s.positions), np.zeros_like(s.positions), 1.0, 10)
    assert abs(res["positions_sum_after_10_steps"] - x.sum()) <= 1e-9 * x.size
