"""A continuous-batching MD server on one GPU.

Requests (a Lumol system and a number of Velocity-Verlet steps) arrive over
time.  The server keeps their state resident on the device:

* a lane is one engine holding a batch of requests on its own CUDA stream,
  stepped by its own host thread in chunks of `chunk` steps; lanes step
  independently (a lane never waits for another one), so the work of requests
  admitted at different times overlaps on the device;
* an arriving request joins the least loaded lane with room (lg_add_systems:
  the requests already there keep their device state and continue), or opens
  a new lane while there are fewer than `max_lanes`; it is admitted only when
  its estimated device footprint fits in the free HBM (cudaMemGetInfo) minus a
  reserve, and in the optional memory budget; otherwise it waits;
* between two chunks a lane retires the requests that finished (their state is
  read back and they leave in place with lg_remove_system, which allocates
  nothing), takes in the requests that joined, drops cancelled ones and takes
  snapshots;
* a request whose state becomes non-finite (the reference panics there,
  lumol-core/src/sys/compute.rs:125,141) fails alone: the engine flags it
  (lg_system_status), it leaves its lane with an error, and the other
  requests of the lane continue from the same chunk.

Each system's arithmetic depends only on its own atoms (per-atom gathers,
per-system list rebuilds and reductions, a fixed group width per atom), so a
request gives the same result alone and in the mix, within the stated
tolerance (tests/test_gpu_serving.py).
"""
from __future__ import annotations

import ctypes
import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _capi as C
from .system import Engine, System, VelocityVerlet, md_params


@dataclass
class Request:
    rid: int
    system: System
    nsteps: int
    timestep: float
    arrival: float = 0.0          # seconds after the server started
    kind: str = ""
    # a snapshot to resume from: (positions, velocities, accelerations, steps done)
    restore: tuple | None = None
    # filled by the server
    admitted: float | None = None
    finished: float | None = None
    steps_done: int = 0
    positions: np.ndarray | None = None
    velocities: np.ndarray | None = None
    error: str | None = None
    cancelled: bool = False
    snapshot: tuple | None = None  # (positions, velocities, accelerations, steps done), on request

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def footprint_bytes(system: System, precision: str, skin: float = 1.0) -> int:
    """Device bytes a system needs in an engine (per-atom state, neighbour list
    at the engine's capacity rule, Ewald tables), used for admission."""
    n = system.size
    rc = max([p.cutoff for p in system.pairs.values()] + [system.coulomb.cutoff if system.coulomb else 0.0])
    rlist = rc + skin
    density = n / system.cell.volume()
    maxnb = min(n, int(math.ceil(1.6 * density * 4.0 / 3.0 * math.pi * rlist ** 3 + 64)))
    maxnb = max(32, (maxnb + 31) // 32 * 32)
    per_atom = 4 * 32 + 3 * 24 + 14 * 8 + 16 + 6 * 4 + 4 * maxnb + (32 if precision == "mixed" else 0)
    nk = 0
    kbytes = 0
    if system.coulomb is not None and hasattr(system.coulomb, "kmax"):
        kmax = system.coulomb.kmax
        nk = 4 * kmax ** 3 + 6 * kmax ** 2 + 3 * kmax
        kbytes = nk * (112 + 56 + 32 + 16) + (kmax + 1) * 3 * n * 24 + (nk // 8 + 1) * 3 * n * 8
    return n * per_atom + kbytes + (1 << 20)


def lane_class(system) -> str:
    """The lanes a request may join: "pairs" for systems with pair potentials
    only (no Coulomb, bonds or restrictions: a mixed-precision batch of them
    runs MD in one persistent launch per chunk), "general" for the others, so
    that one Coulomb request does not move a lane of pair fluids onto the
    general per-step kernels."""
    if getattr(system, "coulomb", None) is not None or getattr(system, "bonds", None):
        return "general"
    for p in getattr(system, "pairs", {}).values():
        r = p.restriction
        if (r[0] if isinstance(r, tuple) else r) != 0:
            return "general"
    return "pairs"


class Lane:
    """One engine holding a batch of requests, stepped by its own thread.

    The server thread only appends to `joining`, `cancel` and `snap` (under
    `lock`); everything else, the engine included, belongs to the lane's
    thread."""

    def __init__(self, server: "Server", first: list[Request], cls: str = "general"):
        self.server = server
        self.cls = cls
        self.requests: list[Request] = []
        self.engine = None
        self.joining: list[Request] = list(first)
        self.cancel: set[int] = set()
        self.snap: set[int] = set()
        self.lock = threading.Lock()
        self.open = True           # accepts joins; closed by its thread when it runs empty
        self.atoms = sum(r.system.size for r in first)
        self.members = {r.rid for r in first}  # every request assigned to the lane and not yet gone
        self.thread = threading.Thread(target=self._serve, daemon=True)

    # ---- called by the server thread --------------------------------------------------
    def try_join(self, r: Request) -> bool:
        with self.lock:
            if not self.open:
                return False
            self.joining.append(r)
            self.members.add(r.rid)
            self.atoms += r.system.size
            return True

    def holds(self, rid: int) -> bool:
        with self.lock:
            return rid in self.members

    # ---- the lane's own thread ---------------------------------------------------------
    def _take_joins(self) -> None:
        with self.lock:
            joins, self.joining = self.joining, []
        if not joins:
            return
        if self.engine is None:
            self.engine = self.server.make_engine(len(joins))
            first = 0
        else:
            first = len(self.requests)
            self.engine.call("lg_add_systems", len(joins))
        eng = self.engine
        for k, r in enumerate(joins):  # every new system described before any state is set
            r.system._lower_into(eng, first + k)
        for k, r in enumerate(joins):
            s = first + k
            p = md_params(VelocityVerlet(r.timestep))
            eng.call("lg_md_setup_ex", s, ctypes.byref(p))
            if r.restore is not None:
                x, v, a, done = r.restore
                r.steps_done = int(done)
                eng.call("lg_md_set_state_ex", s, C.dptr(np.ascontiguousarray(x, dtype=np.float64)),
                         C.dptr(np.ascontiguousarray(v, dtype=np.float64)),
                         C.dptr(np.ascontiguousarray(a, dtype=np.float64)))
            else:
                v = r.system.velocities if r.system.velocities is not None else np.zeros((r.system.size, 3))
                eng.call("lg_md_set_state", s, C.dptr(np.ascontiguousarray(r.system.positions, dtype=np.float64)),
                         C.dptr(np.ascontiguousarray(v, dtype=np.float64)))
        with self.lock:
            self.requests += joins
        self.server.stats.joins += len(joins)

    def _state(self, s: int, with_acc: bool = False):
        n = self.requests[s].system.size
        x, v = np.zeros((n, 3)), np.zeros((n, 3))
        a = np.zeros((n, 3)) if with_acc else None
        self.engine.call("lg_md_get_state_ex", s, C.dptr(x), C.dptr(v), C.dptr(a) if with_acc else None)
        return x, v, a

    def _leave(self, indices: list[int]) -> None:
        for s in sorted(indices, reverse=True):
            with self.lock:
                r = self.requests[s]
                last = len(self.requests) == 1
            if not last:
                self.engine.call("lg_remove_system", s)
                self.server.stats.leaves += 1
            else:  # the engine keeps at least one system: it closes with its last one
                self.engine.close()
                self.engine = None
            with self.lock:
                del self.requests[s]
                self.members.discard(r.rid)
                self.atoms -= r.system.size

    def _boundary(self) -> None:
        """Snapshots, cancellation and retirement between two chunks."""
        now = self.server.now()
        leave = []
        with self.lock:
            cancel, self.cancel = self.cancel, set()
            snap, self.snap = self.snap, set()
        for s, r in enumerate(self.requests):
            if r.rid in snap and r.error is None:
                x, v, a = self._state(s, with_acc=True)
                r.snapshot = (x, v, a, r.steps_done)
            if r.error is not None:
                leave.append(s)
            elif r.rid in cancel:
                r.cancelled = True
                r.finished = now
                leave.append(s)
            elif r.steps_done >= r.nsteps:
                r.positions, r.velocities, _ = self._state(s)
                r.finished = now
                leave.append(s)
        present = {r.rid for r in self.requests}
        with self.lock:  # controls of requests still joining wait for their first boundary
            self.cancel |= {rid for rid in cancel if rid not in present}
            self.snap |= {rid for rid in snap if rid not in present}
        done = [self.requests[s] for s in leave]
        if leave:
            self._leave(leave)
        for r in done:
            self.server._complete(r)

    def _run_chunk(self) -> None:
        steps = max(0, min(self.server.chunk, min(r.nsteps - r.steps_done for r in self.requests)))
        t0 = time.perf_counter()
        code = self.engine.run_steps(steps)
        self.server.stats.run_s += time.perf_counter() - t0
        if code == C.LG_ERR_NONFINITE:  # the flagged requests fail; the others completed the chunk
            flags = (ctypes.c_uint32 * len(self.requests))()
            self.engine.call("lg_system_status", flags, 1)
            for s, r in enumerate(self.requests):
                if flags[s] & C.LG_SYS_NONFINITE:
                    r.error = "non-finite positions or velocities (Kinetic energy is infinite!)"
                    r.finished = self.server.now()
                    self.server.stats.failed += 1
        elif code != C.LG_OK:
            self.engine.check(code)
        for r in self.requests:
            if r.error is None:
                r.steps_done += steps
                self.server.stats.atom_steps += steps * r.system.size
        self.server.stats.chunks += 1

    def _serve(self) -> None:
        try:
            while True:
                t0 = time.perf_counter()
                self._take_joins()
                self.server.stats.join_s += time.perf_counter() - t0
                if not self.requests:
                    with self.lock:
                        if not self.joining:
                            self.open = False
                            break
                    continue
                # requests that joined or were controlled before their first chunk
                t0 = time.perf_counter()
                self._boundary()
                self.server.stats.boundary_s += time.perf_counter() - t0
                if self.requests:
                    self._run_chunk()
                    t0 = time.perf_counter()
                    self._boundary()
                    self.server.stats.boundary_s += time.perf_counter() - t0
        except BaseException as exc:  # a lane that fails reports every request it holds
            with self.lock:
                self.open = False
                pending = self.requests + self.joining
                self.requests, self.joining = [], []
            for r in pending:
                if r.finished is None:
                    r.error = f"lane failed: {exc!r}"
                    r.finished = self.server.now()
                    self.server._complete(r)
            if self.engine is not None:
                self.engine.close()
                self.engine = None


@dataclass
class ServerStats:
    chunks: int = 0
    lanes_opened: int = 0
    max_lanes: int = 0
    joins: int = 0
    leaves: int = 0
    waited_for_memory: int = 0
    failed: int = 0
    atom_steps: int = 0
    # host seconds the lane threads spent (summed over lanes): taking in joins
    # (description lowering), running chunks (device work + the first run's
    # re-lowering after a change), retiring at boundaries (state reads, leaves)
    join_s: float = 0.0
    run_s: float = 0.0
    boundary_s: float = 0.0


class Server:
    """Continuous batching of MD requests on one GPU."""

    def __init__(self, precision: str = "mixed", chunk: int = 50, max_lanes: int = 4,
                 memory_budget: int | None = None, reserve_bytes: int = 1 << 30, threads_per_atom: int = 8,
                 lane_atoms: int = 400_000, engine_factory=None, free_bytes=None):
        """`engine_factory(n_systems, precision, threads_per_atom)` and
        `free_bytes()` default to the GPU engine and cudaMemGetInfo; the CPU
        tests of the scheduling logic pass stand-ins."""
        self.engine_factory = engine_factory or (lambda n, prec, tpa: Engine(n, prec, threads_per_atom=tpa))
        self.device_free = free_bytes or _device_free_bytes
        self.precision = precision
        self.chunk = chunk
        self.max_lanes = max_lanes
        self.memory_budget = memory_budget
        self.reserve = reserve_bytes
        self.tpa = threads_per_atom
        self.lane_atoms = lane_atoms
        self.lanes: list[Lane] = []
        self.stats = ServerStats()
        self._done: queue.Queue = queue.Queue()
        self._t0 = time.perf_counter()
        self._active: dict[int, Request] = {}
        self._lock = threading.Lock()

    def now(self) -> float:
        return time.perf_counter() - self._t0

    def make_engine(self, n_systems: int):
        return self.engine_factory(n_systems, self.precision, self.tpa)

    def _complete(self, r: Request) -> None:
        with self._lock:
            self._active.pop(r.rid, None)
        self._done.put(r)

    # ---- controls -------------------------------------------------------------------
    def cancel(self, rid: int) -> bool:
        """Stops request `rid` at its lane's next chunk boundary."""
        for lane in list(self.lanes):
            if lane.holds(rid):
                with lane.lock:
                    lane.cancel.add(rid)
                return True
        return False

    def snapshot(self, rid: int) -> bool:
        """Asks for request `rid`'s state at its lane's next chunk boundary
        (Request.snapshot; resume it with Request(restore=snapshot))."""
        for lane in list(self.lanes):
            if lane.holds(rid):
                with lane.lock:
                    lane.snap.add(rid)
                return True
        return False

    # ---- admission --------------------------------------------------------------------
    def _free_bytes(self) -> int:
        free = self.device_free() - self.reserve
        if self.memory_budget is not None:
            with self._lock:
                used = sum(footprint_bytes(r.system, self.precision) for r in self._active.values())
            free = min(free, self.memory_budget - used)
        return free

    def _admit(self, waiting: list[Request]) -> list[Request]:
        now = self.now()
        self.lanes = [lane for lane in self.lanes if lane.open or lane.thread.is_alive()]
        rest = []
        free = None
        for r in waiting:
            if r.arrival > now:
                rest.append(r)
                continue
            if free is None:
                free = self._free_bytes()
            need = footprint_bytes(r.system, self.precision)
            if need > free:
                self.stats.waited_for_memory += 1
                rest.append(r)
                continue
            # a new lane of the request's class while that class has fewer than
            # max_lanes (lanes step concurrently), else the least loaded lane of
            # the class with room
            cls = lane_class(r.system)
            mine = [l for l in self.lanes if l.open and l.cls == cls]
            placed = False
            if len(mine) < self.max_lanes:
                lane = Lane(self, [r], cls)
                self.lanes.append(lane)
                self.stats.lanes_opened += 1
                lane.thread.start()
                placed = True
            else:
                for lane in sorted(mine, key=lambda l: l.atoms):
                    if lane.atoms + r.system.size <= self.lane_atoms and lane.try_join(r):
                        placed = True
                        break
            if not placed:
                rest.append(r)
                continue
            r.admitted = now
            with self._lock:
                self._active[r.rid] = r
            free -= need
        self.stats.max_lanes = max(self.stats.max_lanes, len([l for l in self.lanes if l.open]))
        return rest

    # ---- the loop ---------------------------------------------------------------------
    def run(self, requests: list[Request], on_start=None) -> list[Request]:
        """Serves `requests` (arrival times in seconds from now) and returns
        them completed (finished, cancelled or failed), in completion order.
        `on_start(server)`, if given, runs once the first requests are admitted
        (tests use it to cancel or snapshot requests while they run)."""
        self._t0 = time.perf_counter()
        waiting = sorted(requests, key=lambda r: r.arrival)
        completed: list[Request] = []
        total = len(requests)
        started = False
        while len(completed) < total:
            if waiting:
                waiting = self._admit(waiting)
                if waiting and not self._active and not any(l.open for l in self.lanes):
                    if all(r.arrival <= self.now() for r in waiting):
                        r0 = waiting[0]
                        raise RuntimeError(
                            "a request's device footprint exceeds the memory available to the server "
                            f"(request {r0.rid}: {footprint_bytes(r0.system, self.precision)} bytes; "
                            f"free {self._free_bytes()} bytes after a reserve of {self.reserve})")
            if not started and self._active and on_start is not None:
                started = True
                on_start(self)
            # wait for a completion, or until the next arrival
            timeout = 0.002
            if waiting:
                timeout = max(0.0005, min(0.05, waiting[0].arrival - self.now()))
            try:
                completed.append(self._done.get(timeout=timeout))
                while True:
                    completed.append(self._done.get_nowait())
            except queue.Empty:
                pass
        for lane in self.lanes:
            lane.thread.join()
        self.lanes = []
        return completed

    def close(self) -> None:
        for lane in self.lanes:
            lane.thread.join()
        self.lanes = []


def _device_free_bytes() -> int:
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


def latency_percentiles(requests: list[Request]) -> tuple[float, float]:
    lat = np.array([r.latency for r in requests if r.error is None and not r.cancelled])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
