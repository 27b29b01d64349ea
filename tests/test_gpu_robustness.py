"""Host synchronisation and failure isolation on the GPU.

* lg_md_propagate / lg_md_integrate keep the state resident on the device and
  upload the host arrays only when they changed (the lazy synchronisation
  behind Integrator::integrate, lumol-sim/src/md/integrators.rs:44-69, and
  MolecularDynamics::propagate, md/molecular_dynamics.rs:66-76): trajectories
  with a copy back every step, every few steps, or only at the end are the
  same, and a host-side change between calls is picked up.
* A system whose state becomes non-finite is flagged alone (the reference
  panics there, sys/compute.rs:125,141): the other systems of the batch finish
  their steps with the results they have alone.
* A list build that finds inconsistent cell counts (what an interrupted build
  leaves) writes nothing out of range; the engine recounts and the results are
  unchanged.  The failure is made on the host (lg_test_stale_cell_counts).
"""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
from lumol_gb300.batch import Batch
import oracle
from lumol_gb300 import _capi as C
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu


def _md_engine(system, dt=1.0):
    eng = system.engine()
    p = lg.md_params(lg.VelocityVerlet(dt))
    eng.call("lg_md_setup_ex", 0, ctypes.byref(p))
    return eng


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lazy_host_sync_gives_the_same_trajectory(precision):
    # argon FCC, 500 atoms, shifted LJ at 10 A (the argon MD workload)
    a = workloads.argon_fcc(precision=precision)
    b = workloads.argon_fcc(precision=precision)
    ea, eb = _md_engine(a), _md_engine(b)
    xa, va = a.positions.copy(), a.velocities.copy()
    xb, vb = b.positions.copy(), b.velocities.copy()
    for step in range(20):  # Integrator::integrate once per step, copied back every step
        ea.call("lg_md_integrate", C.dptr(xa), C.dptr(va), 1)
    for step in range(20):  # copied back every 5 steps only (an output cadence)
        flags = C.LG_SYNC_DOWNLOAD if (step + 1) % 5 == 0 else 0
        eb.call("lg_md_propagate", C.dptr(xb), C.dptr(vb), 1, flags)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    # the FP64 trajectory is the oracle's
    if precision == "fp64":
        orc = oracle.Oracle(workloads.argon_fcc())
        x0 = workloads.argon_fcc()
        xo, vo, _ = orc.velocity_verlet(x0.positions, x0.velocities, np.zeros_like(xa), 1.0, 20)
        assert np.abs(xa - xo).max() < 1e-9


def test_host_change_between_calls_is_uploaded():
    """A host-side edit of the velocities (as a host thermostat would make)
    between two calls is seen by the next call; an unchanged host copy is not
    uploaded again, and the run continues from the device state."""
    s = workloads.argon_fcc()
    eng = _md_engine(s)
    x, v = s.positions.copy(), s.velocities.copy()
    eng.call("lg_md_integrate", C.dptr(x), C.dptr(v), 3)
    v *= 0.5  # host edit
    eng.call("lg_md_integrate", C.dptr(x), C.dptr(v), 2)
    # the oracle: 3 steps, halve the velocities, 2 steps (accelerations carried over)
    orc = oracle.Oracle(workloads.argon_fcc())
    s0 = workloads.argon_fcc()
    xo, vo, ao = orc.velocity_verlet(s0.positions, s0.velocities, np.zeros((s0.size, 3)), 1.0, 3)
    xo, vo, ao = orc.velocity_verlet(xo, vo * 0.5, ao, 1.0, 2)
    assert np.abs(x - xo).max() < 1e-9
    assert np.abs(v - vo).max() < 1e-12


def test_nonfinite_system_fails_alone():
    systems = [workloads.lj_replica(n, rho, 200.0, seed=40 + k) for k, (n, rho) in
               enumerate([(300, 0.5), (216, 0.7), (400, 0.4)])]
    alone = []
    for k in range(3):
        solo = workloads.lj_replica(*[(300, 0.5), (216, 0.7), (400, 0.4)][k], 200.0, seed=40 + k)
        bb = Batch([solo], threads_per_atom=8)
        bb.md_setup([1.0])
        bb.md_run(30)
        alone.append(bb.state(0))
        bb.engine.close()
    pos = systems[1].positions.copy()
    pos[7] = np.nan  # a corrupted request, injected on the host
    systems[1].positions = pos
    batch = Batch(systems, threads_per_atom=8)
    batch.md_setup([1.0, 1.0, 1.0])
    with pytest.raises(lg.EngineError) as err:
        batch.md_run(30)
    assert err.value.code == C.LG_ERR_NONFINITE
    assert "system 1" in str(err.value)
    flags = (ctypes.c_uint32 * 3)()
    batch.engine.call("lg_system_status", flags, 1)
    assert list(flags) == [0, C.LG_SYS_NONFINITE, 0]
    for k in (0, 2):
        x, v = batch.state(k)
        assert np.abs(x - alone[k][0]).max() < 1e-9 and np.abs(v - alone[k][1]).max() < 1e-12
    # the flags were cleared; the healthy systems run on without error once
    # the corrupted one is replaced by a finite state
    x1, v1 = systems[1].positions.copy(), np.zeros((systems[1].size, 3))
    x1[7] = x1[6] + 1.5
    batch.engine.call("lg_md_set_state", 1, C.dptr(np.ascontiguousarray(x1)), C.dptr(v1))
    batch.md_run(5)
    batch.engine.call("lg_system_status", flags, 0)
    assert list(flags) == [0, 0, 0]
    batch.engine.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stale_cell_counts_are_recounted(precision):
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5, precision=precision)
    f0, e0, w0 = s.compute()
    eng = s.engine()
    eng.call("lg_test_stale_cell_counts", 0, 1000)
    f1, e1, w1 = s.compute()
    assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0)


def test_stale_cell_counts_in_persistent_md():
    """The persistent kernel's list build finds the stale counts, stops the
    group before using the list, and the chunk is replayed after a recount:
    the trajectory is the one without the injection (every system's lists are
    rebuilt at the replay, which the mixed path's compensated force sums leave
    unchanged up to the last bits)."""
    def make():
        systems, _, _ = workloads.lj_replicas(count=6, seed=11, precision="mixed")
        b = Batch(systems, precision="mixed", threads_per_atom=8)
        b.md_setup([1.0] * len(systems))
        return b
    ref, hit = make(), make()
    ref.md_run(32)
    hit.md_run(8)
    hit.engine.call("lg_test_stale_cell_counts", 2, 50)
    hit.md_run(24)
    for k in range(6):
        xr, vr = ref.state(k)
        xh, vh = hit.state(k)
        assert np.abs(xr - xh).max() < 1e-7 and np.abs(vr - vh).max() < 1e-9
    ref.engine.close()
    hit.engine.close()
