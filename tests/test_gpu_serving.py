"""The continuous-batching server: requests admitted while others run, their
work overlapping on the device, each result the same alone and in the mix.

Stated tolerance: final positions of a request served in the mix and the same
request run alone in its own engine agree within 1e-9 A (FP64)."""
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
    assert server.stats.max_lanes >= 2          # requests overlapped on the device
    for r in done:
        pos, vel = run_alone(r, "fp64", 8)
        assert np.abs(r.positions - pos).max() < 1e-9, r.rid
        assert np.abs(r.velocities - vel).max() < 1e-9, r.rid
    p50, p99 = latency_percentiles(done)
    assert 0.0 < p50 <= p99


def test_served_mixed_results_are_alone_results_bit_for_bit():
    """Mixed precision, pair-potential requests: the server runs its lanes in
    chunks of 20 steps through the persistent kernel, a request alone runs in
    launches of 32 steps; every step's arithmetic is the same in both, so the
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
