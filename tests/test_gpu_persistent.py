"""Persistent batched MD (one launch per run of steps, one thread-block cluster
per group of systems) against the per-step kernels of the same mixed path.

The two paths share the force arithmetic (every FP32 rounding written out),
the order of every force sum, the neighbour-list builder's entry order and the
Berendsen factor's kinetic-energy sums, so their trajectories are the same bit
for bit, list rebuilds and thermostats included.
"""
import ctypes

import numpy as np
import pytest

from lumol_gb300 import workloads
from lumol_gb300.batch import Batch

pytestmark = pytest.mark.gpu

PARAMS = [(64, 0.4, 120.0), (4096, 0.85, 90.0), (900, 0.3, 280.0), (1500, 0.7, 200.0), (300, 0.9, 150.0),
          (2500, 0.5, 110.0), (128, 0.6, 250.0)]


def replicas():
    return [workloads.lj_replica(n, rho, t, 700 + k, "mixed") for k, (n, rho, t) in enumerate(PARAMS)]


def launches(batch):
    count = ctypes.c_uint64()
    batch.engine.call("lg_launch_count", ctypes.byref(count))
    return count.value


def run(persistent, thermostats, calls, tpa=4, staging=False):
    """Both paths with the same threads per atom, so every force sum runs in the same order."""
    systems = replicas()
    batch = Batch(systems, precision="mixed", persistent=persistent, threads_per_atom=tpa, staging=staging)
    batch.md_setup([1.0] * len(systems), thermostats)
    for k in calls:
        before = launches(batch)
        batch.md_run(k)
        if persistent and k >= 4:  # one launch per run of up to 256 steps (shorter runs: per-step
            # kernels), each with the one-thread kernel that hands the status word to the host
            assert launches(batch) - before == 2 * ((k + 255) // 256)
    out = [batch.state(s) for s in range(len(systems))]
    batch.engine.close()
    return out


@pytest.mark.parametrize("thermo,tpa", [(False, 4), (True, 4), (True, 1), (True, 2)])
def test_persistent_matches_per_step_kernels(thermo, tpa):
    thermostats = [(t, 100.0) if (thermo and k % 2 == 0) else None for k, (n, rho, t) in enumerate(PARAMS)]
    calls = [1, 40, 7, 300]  # run lengths across and inside the 256-step launches
    a = run(True, thermostats, calls, tpa)
    b = run(False, thermostats, calls, tpa)
    for (pa, va), (pb, vb) in zip(a, b):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_staged_positions_match_per_step_kernels():
    """LG_OPT_STAGING: every block copies its group's fixed-point positions into
    shared memory each step and gathers neighbours from there; the
    trajectories are the per-step kernels' bit for bit."""
    thermostats = [(t, 100.0) if k % 2 == 0 else None for k, (n, rho, t) in enumerate(PARAMS)]
    calls = [40, 300]
    a = run(True, thermostats, calls, 2, staging=True)
    b = run(False, thermostats, calls, 2)
    for (pa, va), (pb, vb) in zip(a, b):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_persistent_rebuilds_lists():
    """Hot, dilute replicas over 200 steps: every system rebuilds its list
    several times inside the persistent launches, and the trajectories stay
    the same bit for bit."""
    systems = replicas()
    batch = Batch(systems, precision="mixed", threads_per_atom=4)
    batch.md_setup([1.0] * len(systems))
    e0 = [batch.energy(s) for s in range(len(systems))]
    batch.md_run(200)
    ref = Batch(replicas(), precision="mixed", persistent=False, threads_per_atom=4)
    ref.md_setup([1.0] * len(systems))
    ref.md_run(200)
    for s in range(len(systems)):
        pa, va = batch.state(s)
        pb, vb = ref.state(s)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
        assert np.isfinite(e0[s])


@pytest.mark.parametrize("persistent", [False, True])
def test_md_paths_are_deterministic(persistent):
    """The same run twice gives bit-identical positions and velocities: no
    force, list or reduction depends on the order in which threads finish."""
    thermostats = [(t, 100.0) if k % 2 == 0 else None for k, (n, rho, t) in enumerate(PARAMS)]
    a = run(persistent, thermostats, [40, 7])
    b = run(persistent, thermostats, [40, 7])
    for (pa, va), (pb, vb) in zip(a, b):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def clustered_droplet(seed, precision="mixed"):
    """A solid-density argon crystallite (FCC, a = 5.26 A, 864 atoms, LJ cut at
    12 A) in one corner of a box four times wider.  The engine sizes the
    neighbour capacity from each system's mean density, so the crystallite's
    rows (about 250 neighbours within 13 A) overflow the first list build and
    the engine regrows the lists and replays the run."""
    from lumol_gb300 import LennardJones, PairInteraction, System, UnitCell
    from lumol_gb300.units import from_
    rng = np.random.default_rng(seed)
    a, cells = 5.26, 6
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    grid = np.array([[i, j, k] for i in range(cells) for j in range(cells) for k in range(cells)], dtype=float)
    pos = (grid[:, None, :] + base[None, :, :]).reshape(-1, 3) * a + 1.0
    pos = pos + rng.uniform(-0.05, 0.05, size=pos.shape)
    s = System(UnitCell.cubic(4 * cells * a), precision=precision)
    s.add_particles(["Ar"] * len(pos), pos, masses=[39.948] * len(pos))
    lj = LennardJones(sigma=3.405, epsilon=from_(0.996, "kJ/mol"))
    s.set_pair_potential(("Ar", "Ar"), PairInteraction.shifted(lj, 12.0))
    s.velocities = workloads.boltzmann_velocities(s, 40.0, seed + 1)
    return s


def test_persistent_list_overflow_is_regrown_and_replayed():
    def run_once(persistent):
        systems = [clustered_droplet(3), workloads.lj_replica(300, 0.3, 120.0, 9, "mixed")]
        batch = Batch(systems, precision="mixed", persistent=persistent, threads_per_atom=4)
        batch.md_setup([1.0, 1.0])
        batch.md_run(40)
        out = [batch.state(s) for s in range(2)]
        batch.engine.close()
        return out
    a = run_once(True)
    b = run_once(False)
    for (pa, va), (pb, vb) in zip(a, b):
        assert np.all(np.isfinite(pa)) and np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_persistent_other_pair_potentials():
    """Fluids of the Born-Mayer-Huggins, Morse, Gaussian and Mie potentials and
    of TableComputations (plain, shifted and tail-corrected pairs of two kinds) in one batch with
    an LJ replica, two of them under a thermostat: the persistent launches
    give the per-step kernels' trajectories bit for bit."""
    import systems as fluids

    def make():
        out = [fluids.random_lj_fluid(400 + 50 * k, 0.02, 30 + k, 9.0, family=f, precision="mixed")
               for k, f in enumerate(["bmh", "morse", "gaussian", "mie", "table"])]
        return out + [workloads.lj_replica(500, 0.7, 150.0, 77, "mixed")]

    states = []
    for persistent in (True, False):
        systems = make()
        batch = Batch(systems, precision="mixed", persistent=persistent, threads_per_atom=8)
        batch.md_setup([1.0] * len(systems), [None, (200.0, 50.0), None, (150.0, 20.0), None, None])
        batch.md_run(40)
        states.append([batch.state(s) for s in range(len(systems))])
        batch.engine.close()
    for (pa, va), (pb, vb) in zip(*states):
        assert np.all(np.isfinite(pa))
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_pinned_host_buffers_match_pageable():
    """lg_md_set_state(_all) / lg_md_get_state(_all) read and write page-locked
    host buffers in place (the pack kernels take their mapped addresses) and
    stage pageable ones: the trajectories and the returned states are the same
    bit for bit."""
    torch = pytest.importorskip("torch")
    from lumol_gb300 import _capi as C

    def go(pinned):
        systems = replicas()
        n = sum(s.size for s in systems)
        batch = Batch(systems, precision="mixed", threads_per_atom=4)
        batch.md_setup([1.0] * len(systems))
        batch.md_run(1)

        def alloc(rows):
            if pinned:
                return torch.zeros((rows, 3), dtype=torch.float64, pin_memory=True).numpy()
            return np.zeros((rows, 3))

        pos, vel = alloc(n), alloc(n)
        eng = batch.engine
        eng.call("lg_md_get_state_all", C.dptr(pos), C.dptr(vel), None)
        for k in (1, 3, 40):
            eng.call("lg_md_set_state_all", C.dptr(pos), C.dptr(vel), None)
            eng.call("lg_md_run", k)
            eng.call("lg_md_get_state_all", C.dptr(pos), C.dptr(vel), None)
        m = systems[3].size
        p3, v3 = alloc(m), alloc(m)
        eng.call("lg_md_get_state", 3, C.dptr(p3), C.dptr(v3))
        p3 += 0.01
        eng.call("lg_md_set_state", 3, C.dptr(p3), C.dptr(v3))
        eng.call("lg_md_run", 5)
        eng.call("lg_md_get_state", 3, C.dptr(p3), C.dptr(v3))
        out = (pos.copy(), vel.copy(), p3.copy(), v3.copy())
        eng.close()
        return out

    a, b = go(True), go(False)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_autotuned_width_keeps_the_state():
    """A persistent batch without a fixed group size is tuned on trial launches
    of the persistent kernel (1, 2, 4 and 8 threads per atom), each undone from
    the launch's own checkpoint: a zero-step run (which tunes) leaves the
    positions and velocities bit for bit as they were, and the tuned runs stay
    finite and planned on the persistent kernel.  (An atom count no other test
    uses, so the tuning is not taken from the cache.)"""
    params = [(333, 0.6, 150.0), (1201, 0.8, 110.0), (77, 0.5, 200.0)]
    systems = [workloads.lj_replica(n, rho, t, 900 + k, "mixed") for k, (n, rho, t) in enumerate(params)]
    batch = Batch(systems, precision="mixed")
    batch.md_setup([1.0] * len(systems), [(t, 100.0) for _, _, t in params])
    before = [batch.state(s) for s in range(len(systems))]
    batch.md_run(0)
    after = [batch.state(s) for s in range(len(systems))]
    for (pa, va), (pb, vb) in zip(before, after):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    batch.md_run(40)
    cluster, groups = ctypes.c_int32(), ctypes.c_int32()
    batch.engine.call("lg_md_plan", ctypes.byref(cluster), ctypes.byref(groups))
    assert cluster.value > 0 and groups.value > 0
    for s in range(len(systems)):
        p, v = batch.state(s)
        assert np.all(np.isfinite(p)) and np.all(np.isfinite(v))
    batch.engine.close()


def test_one_kind_lj_variant_matches_the_generic_kernels():
    """Batches whose systems all have one kind and a Lennard-Jones pair run
    force loops compiled for that case (per-step and persistent).  The same
    replicas described with two kinds and the same parameters for every pair
    take the generic kernels: forces and 60-step trajectories are equal bit
    for bit."""
    from lumol_gb300 import LennardJones, PairInteraction, System
    from lumol_gb300.units import from_

    def two_kinds(one):
        s = System(one.cell, precision="mixed")
        names = ["Ar" if k % 2 == 0 else "Xr" for k in range(one.size)]
        s.add_particles(names, one.positions, masses=[39.948] * one.size)
        lj = LennardJones(sigma=3.405, epsilon=from_(0.996, "kJ/mol"))
        for pair in (("Ar", "Ar"), ("Ar", "Xr"), ("Xr", "Xr")):
            s.set_pair_potential(pair, PairInteraction.shifted(lj, 2.5 * 3.405))
        s.velocities = one.velocities.copy()
        return s

    params = [(500, 0.7, 120.0), (1200, 0.5, 200.0), (130, 0.8, 150.0)]
    ones = [workloads.lj_replica(n, rho, t, 40 + k, "mixed") for k, (n, rho, t) in enumerate(params)]
    twos = [two_kinds(s) for s in ones]
    for a, b in zip(ones, twos):
        fa, ea, wa = a.compute()
        fb, eb, wb = b.compute()
        assert np.array_equal(fa, fb) and ea == eb and np.array_equal(wa, wb)
    states = []
    for systems in (ones, twos):
        batch = Batch(systems, precision="mixed", threads_per_atom=2)
        batch.md_setup([1.0] * len(systems), [(t, 100.0) for _, _, t in params])
        batch.md_run(60)
        states.append([batch.state(s) for s in range(len(systems))])
        batch.engine.close()
    for (pa, va), (pb, vb) in zip(*states):
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
