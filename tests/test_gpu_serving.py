"""The continuous-batching server: requests admitted while others run, their
work overlapping on the device, each result the same alone and in the mix.

Stated tolerance: final positions of a request served in the mix and the same
request run alone in its own engine agree within 1e-9 A (FP64)."""
import threading
import time

import numpy as np
import pytest

from lumol_gb300 import workloads
from lumol_gb300.batch import Batch
from lumol_gb300.serving import Server, latency_percentiles

pytestmark = pytest.mark.gpu


def run_alone(request, precision, tpa):
    batch = Batch([request.system], precision=precision, threads_per_atom=tpa)
    batch.md_setup([request.timestep])
    batch.md_run(request.nsteps)
    pos, vel = batch.state(0)
    batch.engine.close()
    return pos, vel


def test_served_results_equal_alone_results():
    requests = workloads.serving_requests(count=10, rate=200.0, seed=5, precision="fp64", scale=0.03)
    server = Server(precision="fp64", chunk=20, max_lanes=3, threads_per_atom=8)
    done = server.run(requests)
    server.close()
    assert len(done) == len(requests)
    # requests admitted while others ran: their work overlapped on the device
    assert any(a.admitted < b.finished and b.admitted < a.finished for a in done for b in done if a is not b)
    for r in done:
        pos, vel = run_alone(r, "fp64", 8)
        assert np.abs(r.positions - pos).max() < 1e-9, r.rid
        assert np.abs(r.velocities - vel).max() < 1e-9, r.rid
    p50, p99 = latency_percentiles(done)
    assert 0.0 < p50 <= p99


def test_served_mixed_results_are_alone_results_bit_for_bit():
    """Mixed precision, pair-potential requests: the server runs its lanes in
    chunks of 20 steps through the persistent kernel, a request alone runs in
    launches of up to 256 steps; every step's arithmetic is the same in both, so the
    trajectories are equal bit for bit."""
    requests = [r for r in workloads.serving_requests(count=16, rate=200.0, seed=6, precision="mixed",
                                                      scale=0.03) if r.kind == "lj"]
    assert len(requests) >= 4
    server = Server(precision="mixed", chunk=20, max_lanes=3, threads_per_atom=8)
    done = server.run(requests)
    server.close()
    assert len(done) == len(requests)
    for r in done:
        pos, vel = run_alone(r, "mixed", 8)
        assert np.array_equal(r.positions, pos) and np.array_equal(r.velocities, vel), r.rid


def test_admission_waits_for_memory():
    requests = workloads.serving_requests(count=6, rate=1000.0, seed=9, precision="mixed", scale=0.03)
    for r in requests:
        r.arrival = 0.0  # all at once: they contend for the budget
    from lumol_gb300.serving import footprint_bytes
    biggest = max(footprint_bytes(r.system, "mixed") for r in requests)
    # a budget that holds the biggest request but not all of them at once
    server = Server(precision="mixed", chunk=20, max_lanes=4, memory_budget=int(1.5 * biggest),
                    reserve_bytes=0, threads_per_atom=8)
    done = server.run(requests)
    server.close()
    assert len(done) == len(requests)
    assert server.stats.waited_for_memory > 0


def test_bad_request_fails_alone_and_others_match_alone_runs():
    """A request whose positions hold a NaN (injected on the host) fails with an
    error; the requests served beside it, in the same lanes, finish with their
    alone results."""
    requests = [r for r in workloads.serving_requests(count=12, rate=400.0, seed=8, precision="fp64",
                                                      scale=0.03) if r.kind == "lj"][:5]
    assert len(requests) >= 4
    bad = requests[1]
    pos = bad.system.positions.copy()
    pos[3] = np.nan
    bad.system.positions = pos
    server = Server(precision="fp64", chunk=20, max_lanes=2, threads_per_atom=8)
    done = server.run(requests)
    server.close()
    assert len(done) == len(requests)
    assert bad.error is not None and "non-finite" in bad.error
    assert server.stats.failed == 1
    for r in done:
        if r is bad:
            continue
        assert r.error is None
        pos, vel = run_alone(r, "fp64", 8)
        assert np.abs(r.positions - pos).max() < 1e-9, r.rid


def test_cancel_and_snapshot_restore():
    """A cancelled request leaves at its lane's next boundary; a snapshot taken
    while a request runs, restored as a new request, finishes where the
    uninterrupted run finishes (FP64, 1e-9 A)."""
    requests = [r for r in workloads.serving_requests(count=12, rate=1000.0, seed=12, precision="fp64",
                                                      scale=0.05) if r.kind == "lj"][:3]
    for r in requests:
        r.arrival = 0.0
        r.nsteps = 200
    victim, traced = requests[0], requests[1]

    def control(server):
        server.cancel(victim.rid)

        def later():  # a snapshot once the traced request has run some steps
            t0 = time.perf_counter()
            while traced.steps_done < 40 and time.perf_counter() - t0 < 30.0:
                time.sleep(0.0005)
            server.snapshot(traced.rid)
        threading.Thread(target=later, daemon=True).start()

    server = Server(precision="fp64", chunk=20, max_lanes=2, threads_per_atom=8)
    done = server.run(requests, on_start=control)
    server.close()
    assert victim.cancelled and victim.positions is None
    assert traced.snapshot is not None
    x, v, a, steps = traced.snapshot
    assert 0 < steps < traced.nsteps
    from lumol_gb300.serving import Request
    resumed = Request(rid=99, system=traced.system, nsteps=traced.nsteps, timestep=traced.timestep,
                      restore=(x, v, a, steps))
    server = Server(precision="fp64", chunk=20, max_lanes=1, threads_per_atom=8)
    again = server.run([resumed])
    server.close()
    assert again[0].steps_done == traced.nsteps
    assert np.abs(again[0].positions - traced.positions).max() < 1e-9
    assert np.abs(again[0].velocities - traced.velocities).max() < 1e-9


def test_joining_and_leaving_in_place_keeps_trajectories():
    """Systems join and leave a running engine in place (lg_add_systems,
    lg_remove_system): the systems that stay continue their trajectories
    (FP64, 1e-9 A against each system run alone), and leaving allocates no
    device memory."""
    import ctypes
    import torch
    import lumol_gb300 as lg
    from lumol_gb300 import _capi as C
    sizes, total_steps = [200, 300, 250], [40, 60, 40]

    def make(k):
        return workloads.lj_replica(sizes[k], 0.6, 150.0, seed=70 + k)

    ref = []
    for k in range(3):
        b = Batch([make(k)], threads_per_atom=8)
        b.md_setup([1.0])
        b.md_run(total_steps[k])
        ref.append(b.state(0))
        b.engine.close()
    systems = [make(k) for k in range(3)]

    def join(eng, k, s):
        systems[k]._lower_into(eng, s)
        p = lg.md_params(lg.VelocityVerlet(1.0))
        eng.call("lg_md_setup_ex", s, ctypes.byref(p))
        eng.call("lg_md_set_state", s, C.dptr(np.ascontiguousarray(systems[k].positions)),
                 C.dptr(np.ascontiguousarray(systems[k].velocities)))

    def state(eng, s, n):
        x, v = np.zeros((n, 3)), np.zeros((n, 3))
        eng.call("lg_md_get_state", s, C.dptr(x), C.dptr(v))
        return x, v

    eng = lg.Engine(2, "fp64", threads_per_atom=8)
    systems[0]._lower_into(eng, 0)
    systems[1]._lower_into(eng, 1)
    join(eng, 0, 0)
    join(eng, 1, 1)
    eng.call("lg_md_run", 20)
    eng.call("lg_add_systems", 1)  # system 2 joins at step 20 of the others
    systems[2]._lower_into(eng, 2)
    join(eng, 2, 2)
    eng.call("lg_md_run", 20)
    x0, v0 = state(eng, 0, 200)
    assert np.abs(x0 - ref[0][0]).max() < 1e-9 and np.abs(v0 - ref[0][1]).max() < 1e-9
    x1, _ = state(eng, 1, 300)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    eng.call("lg_remove_system", 0)  # system 1 becomes 0, system 2 becomes 1
    forces, energy, virial = np.zeros((300, 3)), ctypes.c_double(), np.zeros(9)
    eng.call("lg_compute", 0, C.dptr(x1), C.LG_TERM_ALL, C.LG_WANT_FORCES, C.dptr(forces), ctypes.byref(energy),
             C.dptr(virial))  # the batch is lowered again here, without the system that left
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after >= free_before, (free_before, free_after)
    eng.call("lg_md_run", 20)
    x1, v1 = state(eng, 0, 300)
    assert np.abs(x1 - ref[1][0]).max() < 1e-9 and np.abs(v1 - ref[1][1]).max() < 1e-9
    x2, v2 = state(eng, 1, 250)
    assert np.abs(x2 - ref[2][0]).max() < 1e-9 and np.abs(v2 - ref[2][1]).max() < 1e-9
    eng.close()
