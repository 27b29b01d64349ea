"""Many independent systems in one engine: every kernel launch covers all of
them, and one MD step of the whole batch is one CUDA graph replay."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C
from .system import Engine, System, md_params


class Batch:
    """A batch of Lumol systems evaluated and integrated together on one GPU.

    Each system keeps its own cell, pair table, Coulomb potential, timestep
    and thermostat; atoms are concatenated in system order on the device."""

    def __init__(self, systems: list[System], precision: str = "fp64", skin: float = 1.0,
                 threads_per_atom: int = 0, persistent: bool = True, cluster: int = 0, staging: bool = False):
        self.systems = systems
        self.engine = Engine(len(systems), precision, skin, threads_per_atom=threads_per_atom,
                             persistent=persistent, cluster=cluster, staging=staging)
        for s, system in enumerate(systems):
            system._lower_into(self.engine, s)
        self.offsets = np.cumsum([0] + [s.size for s in systems])

    @property
    def atoms(self) -> int:
        return int(self.offsets[-1])

    def md_setup(self, timesteps=None, thermostats=None, propagators=None) -> None:
        """The MD setup of every system.  Either `timesteps` (VelocityVerlet)
        with thermostats[s] None or a (temperature, tau) Berendsen pair, or
        `propagators`: one MolecularDynamics (integrator, thermostat, controls)
        per system."""
        for s, system in enumerate(self.systems):
            if propagators is not None:
                md = propagators[s]
                p = md_params(md.integrator, md.thermostat, md.controls)
                self.engine.call("lg_md_setup_ex", s, ctypes.byref(p))
                continue
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

    # ---- batched Monte Carlo chains ---------------------------------------------------
    def mc_setup(self, s: int, temperature: float, delta: float, seed: int) -> None:
        """MonteCarlo(temperature) with Translate(delta) moves for system `s`."""
        self.engine.call("lg_mc_setup", s, float(temperature), float(delta), int(seed) & (2 ** 64 - 1))

    def mc_setup_moves(self, s: int, temperature: float, translate=(0.3, 1.0), rotate=None, seed: int = 0) -> None:
        """MonteCarlo(temperature) with Translate(delta) at frequency f_t and
        Rotate(theta) at f_r (`translate` / `rotate` = (amplitude, frequency) or
        None) for system `s`: rigid moves of whole molecules."""
        td, tf = translate if translate else (0.0, 0.0)
        rt, rf = rotate if rotate else (0.0, 0.0)
        self.engine.call("lg_mc_setup_ex", s, float(temperature), float(td), float(tf), float(rt), float(rf),
                         int(seed) & (2 ** 64 - 1))

    def mc_run(self, moves: int) -> None:
        """`moves` attempted moves in every chain."""
        self.engine.call("lg_mc_run", int(moves))

    def mc_stats(self, s: int):
        energy = ctypes.c_double()
        acc, att = ctypes.c_int64(), ctypes.c_int64()
        self.engine.call("lg_mc_stats", s, ctypes.byref(energy), ctypes.byref(acc), ctypes.byref(att))
        return energy.value, acc.value, att.value

    def energy(self, s: int) -> float:
        """Potential energy of system `s` at its current device positions."""
        pos, _ = self.state(s)
        system = self.systems[s]
        out = ctypes.c_double()
        forces = np.zeros((system.size, 3))
        virial = np.zeros(9)
        self.engine.call("lg_compute", s, C.dptr(np.ascontiguousarray(pos)), C.LG_TERM_ALL, C.LG_WANT_ENERGY,
                         C.dptr(forces), ctypes.byref(out), C.dptr(virial))
        return out.value


class SplitMix64:
    """Host copy of the chains' random stream (SplitMix64), for tests that replay
    a chain's moves."""

    def __init__(self, seed: int):
        self.state = (int(seed) * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & (2 ** 64 - 1)

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & (2 ** 64 - 1)
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2 ** 64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2 ** 64 - 1)
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)
