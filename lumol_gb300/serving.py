"""A continuous-batching MD server on one GPU.

Requests (a Lumol system and a number of Velocity-Verlet steps) arrive over
time.  The server keeps their state resident on the device and advances them
in rounds:

* every round, each lane (one engine holding a batch of requests, on its own
  CUDA stream) runs `chunk` steps; lanes run concurrently, so the work of
  requests admitted at different times overlaps on the device;
* at a round boundary, finished requests are read back and retired (a lane
  that lost requests is rebuilt around the remaining ones, carrying positions,
  velocities and accelerations over exactly), and requests that have arrived
  are admitted as a new lane, as long as their estimated device footprint fits
  in the free HBM (cudaMemGetInfo) minus a reserve, and the lane count is below
  its limit; the rest wait;
* small lanes are merged when there are too many of them.

Each system's arithmetic depends only on its own atoms (per-atom gathers,
per-system list rebuilds and reductions), so a request gives the same result
alone and in the mix, within the stated tolerance (tests/test_gpu_serving.py).
"""
from __future__ import annotations

import concurrent.futures
import ctypes
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _capi as C
from .batch import Batch
from .system import System


@dataclass
class Request:
    rid: int
    system: System
    nsteps: int
    timestep: float
    arrival: float = 0.0          # seconds after the server started
    kind: str = ""
    # filled by the server
    admitted: float | None = None
    finished: float | None = None
    steps_done: int = 0
    positions: np.ndarray | None = None
    velocities: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def footprint_bytes(system: System, precision: str, skin: float = 1.0) -> int:
    """Device bytes a system needs in an engine (per-atom state, neighbour list
    at the engine's capacity rule, Ewald tables), used for admission."""
    n = system.size
    L = system.cell.lengths
    rc = max([p.cutoff for p in system.pairs.values()] + [system.coulomb.cutoff if system.coulomb else 0.0])
    rlist = rc + skin
    density = n / (L[0] * L[1] * L[2])
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


class Lane:
    """One engine holding a batch of requests."""

    def __init__(self, requests: list[Request], precision: str, threads_per_atom: int, states=None):
        self.requests = requests
        self.batch = Batch([r.system for r in requests], precision=precision, threads_per_atom=threads_per_atom)
        self.batch.md_setup([r.timestep for r in requests])
        if states is not None:
            pos = np.ascontiguousarray(np.concatenate([s[0] for s in states]))
            vel = np.ascontiguousarray(np.concatenate([s[1] for s in states]))
            acc = np.ascontiguousarray(np.concatenate([s[2] for s in states]))
            self.batch.engine.call("lg_md_set_state_all", C.dptr(pos), C.dptr(vel), C.dptr(acc))

    def states(self):
        n = self.batch.atoms
        pos, vel, acc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        self.batch.engine.call("lg_md_get_state_all", C.dptr(pos), C.dptr(vel), C.dptr(acc))
        off = self.batch.offsets
        return [(pos[off[k]:off[k + 1]], vel[off[k]:off[k + 1]], acc[off[k]:off[k + 1]])
                for k in range(len(self.requests))]

    def steps_left(self) -> int:
        return min(r.nsteps - r.steps_done for r in self.requests)

    def close(self) -> None:
        self.batch.engine.close()


@dataclass
class ServerStats:
    rounds: int = 0
    lane_rebuilds: int = 0
    max_lanes: int = 0
    waited_for_memory: int = 0
    atom_steps: int = 0


class Server:
    """Continuous batching of MD requests on one GPU."""

    def __init__(self, precision: str = "mixed", chunk: int = 50, max_lanes: int = 4,
                 memory_budget: int | None = None, reserve_bytes: int = 1 << 30, threads_per_atom: int = 8):
        self.precision = precision
        self.chunk = chunk
        self.max_lanes = max_lanes
        self.memory_budget = memory_budget
        self.reserve = reserve_bytes
        self.tpa = threads_per_atom
        self.lanes: list[Lane] = []
        self.stats = ServerStats()
        self.pool = concurrent.futures.ThreadPoolExecutor(max_workers=max(2, max_lanes + 1))

    # ---- admission ---------------------------------------------------------------------
    def _free_bytes(self) -> int:
        import torch
        free, _ = torch.cuda.mem_get_info()
        if self.memory_budget is not None:
            used = sum(footprint_bytes(r.system, self.precision) for lane in self.lanes for r in lane.requests)
            free = min(free, self.memory_budget - used)
        return free - self.reserve

    def _admit(self, waiting: list[Request], now: float) -> list[Request]:
        ready = [r for r in waiting if r.arrival <= now]
        if not ready or len(self.lanes) >= self.max_lanes:
            return waiting
        free = self._free_bytes()
        chosen = []
        for r in ready:
            need = footprint_bytes(r.system, self.precision)
            if need <= free:
                chosen.append(r)
                free -= need
            else:
                self.stats.waited_for_memory += 1
        if chosen:
            for r in chosen:
                r.admitted = now
            self.lanes.append(Lane(chosen, self.precision, self.tpa))
        return [r for r in waiting if r not in chosen]

    # ---- retirement and lane maintenance -------------------------------------------------
    def _retire(self, now_fn) -> list[Request]:
        done = []
        new_lanes = []
        for lane in self.lanes:
            finished = [k for k, r in enumerate(lane.requests) if r.steps_done >= r.nsteps]
            if not finished:
                new_lanes.append(lane)
                continue
            states = lane.states()
            t = now_fn()
            for k in finished:
                r = lane.requests[k]
                r.positions, r.velocities = states[k][0].copy(), states[k][1].copy()
                r.finished = t
                done.append(r)
            keep = [k for k in range(len(lane.requests)) if k not in finished]
            lane.close()
            if keep:
                new_lanes.append(Lane([lane.requests[k] for k in keep], self.precision, self.tpa,
                                      [states[k] for k in keep]))
                self.stats.lane_rebuilds += 1
        self.lanes = new_lanes
        return done

    def _merge(self) -> None:
        while len(self.lanes) > self.max_lanes - 1 and len(self.lanes) >= 2:
            self.lanes.sort(key=lambda lane: lane.batch.atoms)
            a, b = self.lanes[0], self.lanes[1]
            reqs = a.requests + b.requests
            states = a.states() + b.states()
            a.close()
            b.close()
            self.lanes = self.lanes[2:] + [Lane(reqs, self.precision, self.tpa, states)]
            self.stats.lane_rebuilds += 1

    # ---- the loop ----------------------------------------------------------------------
    def run(self, requests: list[Request]) -> list[Request]:
        """Serves `requests` (arrival times in seconds from now) and returns
        them completed, in completion order."""
        waiting = sorted(requests, key=lambda r: r.arrival)
        completed: list[Request] = []
        t0 = time.perf_counter()
        now_fn = lambda: time.perf_counter() - t0
        while waiting or self.lanes:
            waiting = self._admit(waiting, now_fn())
            if not self.lanes:
                now = now_fn()
                if all(r.arrival <= now for r in waiting):
                    # nothing runs and nothing arrived could be admitted: it never will be
                    raise RuntimeError("a request's device footprint exceeds the memory available to the server")
                # idle until the next arrival
                time.sleep(max(0.0, min(r.arrival for r in waiting) - now))
                continue
            self.stats.max_lanes = max(self.stats.max_lanes, len(self.lanes))
            steps = [min(self.chunk, lane.steps_left()) for lane in self.lanes]
            futures = [self.pool.submit(lane.batch.md_run, k) for lane, k in zip(self.lanes, steps)]
            for f in futures:
                f.result()
            for lane, k in zip(self.lanes, steps):
                for r in lane.requests:
                    r.steps_done += k
                self.stats.atom_steps += k * lane.batch.atoms
            self.stats.rounds += 1
            completed += self._retire(now_fn)
            self._merge()
        return completed

    def close(self) -> None:
        for lane in self.lanes:
            lane.close()
        self.lanes = []
        self.pool.shutdown()


def latency_percentiles(requests: list[Request]) -> tuple[float, float]:
    lat = np.array([r.latency for r in requests])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
