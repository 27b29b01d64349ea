"""CPU tests of the serving scheduler's host logic, with a stand-in engine.

The stand-in keeps each system's positions on the host and adds the number of
steps run to them, so the tests can follow every request through joins,
leaves, cancellation, snapshots and failures without a GPU.  A request's
"positions" after n steps are therefore its initial positions + n.
"""
import ctypes
import time

import numpy as np
import pytest

from lumol_gb300 import _capi as C
from lumol_gb300.serving import Request, Server


class FakeSystem:
    def __init__(self, n, x0, poison=False):
        self.size = n
        self.positions = np.full((n, 3), float(x0))
        self.velocities = np.zeros((n, 3))
        self.poison = poison

    def _lower_into(self, eng, s):
        eng.describe(s, self)


def _arr(ptr, n):
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double)), shape=(n, 3))


class FakeEngine:
    """The calls a lane makes, on host arrays."""

    def __init__(self, n_systems, log):
        self.sys = [None] * n_systems
        self.x = [None] * n_systems
        self.flags = [0] * n_systems
        self.log = log
        self.closed = False

    def describe(self, s, system):
        self.sys[s] = system

    def call(self, name, *args):
        self.log.append(name)
        if name == "lg_add_systems":
            self.sys += [None] * args[0]
            self.x += [None] * args[0]
            self.flags += [0] * args[0]
        elif name == "lg_remove_system":
            s = args[0]
            del self.sys[s], self.x[s], self.flags[s]
        elif name in ("lg_md_set_state", "lg_md_set_state_ex"):
            s = args[0]
            self.x[s] = _arr(args[1], self.sys[s].size).copy()
        elif name == "lg_md_get_state_ex":
            s = args[0]
            _arr(args[1], self.sys[s].size)[:] = self.x[s]
            if args[3] is not None:
                _arr(args[3], self.sys[s].size)[:] = 0.0
        elif name == "lg_system_status":
            for s, f in enumerate(self.flags):
                args[0][s] = f
            if args[1]:
                self.flags = [0] * len(self.flags)

    def run_steps(self, steps):
        time.sleep(0.002)  # a chunk takes time, as on the device
        bad = False
        for s, system in enumerate(self.sys):
            self.x[s] += steps
            if system.poison:
                self.x[s][:] = np.nan
                self.flags[s] = C.LG_SYS_NONFINITE
                bad = True
        return C.LG_ERR_NONFINITE if bad else C.LG_OK

    def check(self, code):
        C.check(code)

    def close(self):
        self.closed = True


def make_server(log, engines=None, **kw):
    def factory(n, precision, tpa):
        e = FakeEngine(n, log)
        if engines is not None:
            engines.append(e)
        return e
    kw.setdefault("free_bytes", lambda: 1 << 40)
    kw.setdefault("reserve_bytes", 0)
    return Server(precision="fp64", engine_factory=factory, **kw)


def requests(count, nsteps=100, arrival=0.0, sizes=None):
    sizes = sizes or [10 + 3 * k for k in range(count)]
    return [Request(rid=k, system=FakeSystem(sizes[k], 100 * k), nsteps=nsteps, timestep=1.0, arrival=arrival)
            for k in range(count)]


def footprint_stub(monkeypatch, size_bytes=1000):
    import lumol_gb300.serving as srv
    monkeypatch.setattr(srv, "footprint_bytes", lambda system, precision, skin=1.0: size_bytes * system.size)


def test_every_request_finishes_with_its_own_steps(monkeypatch):
    footprint_stub(monkeypatch)
    log, engines = [], []
    reqs = requests(9, nsteps=95)
    for k, r in enumerate(reqs):
        r.nsteps = 200 + 13 * k
        r.arrival = 0.0 if k < 3 else 0.01  # the later ones join running lanes
    server = make_server(log, engines, chunk=20, max_lanes=3)
    done = server.run(reqs)
    assert sorted(r.rid for r in done) == list(range(9))
    for r in done:
        assert r.error is None and not r.cancelled
        assert np.all(r.positions == 100 * r.rid + r.nsteps), r.rid
    assert server.stats.max_lanes == 3 and server.stats.joins == 9
    assert "lg_add_systems" in log and "lg_remove_system" in log  # requests joined and left in place
    # every request leaves in place, except the last one of an engine, which closes it
    assert all(e.closed for e in engines)
    assert server.stats.leaves + len(engines) == 9


def test_cancel_and_snapshot_are_applied_at_the_next_boundary(monkeypatch):
    footprint_stub(monkeypatch)
    log = []
    reqs = requests(3, nsteps=200)
    server = make_server(log, chunk=20, max_lanes=1)

    def control(s):
        assert s.cancel(0)
        assert s.snapshot(1)

    done = server.run(reqs, on_start=control)
    assert len(done) == 3
    assert reqs[0].cancelled and reqs[0].positions is None
    x, v, a, steps = reqs[1].snapshot
    assert steps < 200 and np.all(x == 100 + steps)
    assert np.all(reqs[1].positions == 100 + 200) and np.all(reqs[2].positions == 200 + 200)


def test_restore_resumes_from_the_snapshot(monkeypatch):
    footprint_stub(monkeypatch)
    system = FakeSystem(10, 0.0)
    r = Request(rid=5, system=system, nsteps=100, timestep=1.0,
                restore=(np.full((10, 3), 60.0), np.zeros((10, 3)), np.zeros((10, 3)), 60))
    server = make_server([], chunk=16)
    done = server.run([r])
    assert done[0].steps_done == 100 and np.all(done[0].positions == 100.0)


def test_nonfinite_request_fails_alone(monkeypatch):
    footprint_stub(monkeypatch)
    reqs = requests(4, nsteps=60)
    reqs[2].system.poison = True
    server = make_server([], chunk=20, max_lanes=1)
    done = server.run(reqs)
    assert len(done) == 4
    assert reqs[2].error is not None and "non-finite" in reqs[2].error
    assert server.stats.failed == 1
    for k in (0, 1, 3):
        assert reqs[k].error is None and np.all(reqs[k].positions == 100 * k + 60)


def test_admission_waits_for_memory(monkeypatch):
    footprint_stub(monkeypatch, size_bytes=1000)
    reqs = requests(5, nsteps=40, sizes=[100] * 5)
    # room for two requests at a time
    server = make_server([], chunk=20, max_lanes=4, memory_budget=250_000)
    done = server.run(reqs)
    assert len(done) == 5 and all(r.error is None for r in done)
    assert server.stats.waited_for_memory > 0


def test_request_that_never_fits_is_an_error(monkeypatch):
    footprint_stub(monkeypatch, size_bytes=1000)
    server = make_server([], chunk=20, memory_budget=5_000)
    with pytest.raises(RuntimeError, match="exceeds the memory"):
        server.run(requests(1, sizes=[100]))
