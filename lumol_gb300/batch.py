"""Many independent systems in one engine: every kernel launch covers all of
them, and one MD step of the whole batch is one CUDA graph replay."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C
from .system import Engine, System


class Batch:
    """A batch of Lumol systems evaluated and integrated together on one GPU.

    Each system keeps its own cell, pair table, Coulomb potential, timestep
    and thermostat; atoms are concatenated in system order on the device."""

    def __init__(self, systems: list[System], precision: str = "fp64", skin: float = 1.0):
        self.systems = systems
        self.engine = Engine(len(systems), precision, skin)
        for s, system in enumerate(systems):
            system._lower_into(self.engine, s)
        self.offsets = np.cumsum([0] + [s.size for s in systems])

    @property
    def atoms(self) -> int:
        return int(self.offsets[-1])

    def md_setup(self, timesteps, thermostats=None) -> None:
        """VelocityVerlet::setup for every system; thermostats[s] is None or a
        (temperature, tau) Berendsen pair."""
        for s, system in enumerate(self.systems):
            T0, tau = (thermostats[s] if thermostats and thermostats[s] else (0.0, 0.0))
            self.engine.call("lg_md_setup", s, float(timesteps[s]), float(T0), float(tau))
        for s, system in enumerate(self.systems):
            v = system.velocities if system.velocities is not None else np.zeros((system.size, 3))
            self.engine.call("lg_md_set_state", s, C.dptr(np.ascontiguousarray(system.positions)),
                             C.dptr(np.ascontiguousarray(v, dtype=np.float64)))

    def md_run(self, nsteps: int) -> None:
        self.engine.call("lg_md_run", int(nsteps))

    def state(self, s: int):
        n = self.systems[s].size
        pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
        self.engine.call("lg_md_get_state", s, C.dptr(pos), C.dptr(vel))
        return pos, vel
