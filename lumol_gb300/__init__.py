"""lumol_gb300 -- a GB300 (sm_103a) engine for Lumol's force / energy /
virial / integration path, behind a C ABI (include/lumol_gb300.h).

The Python classes mirror lumol-core / lumol-sim (System, PairInteraction,
LennardJones, Buckingham, Harmonic, Ewald, Wolf, VelocityVerlet,
BerendsenThermostat, MolecularDynamics); every computation runs in the CUDA
library `liblumol_gb300.so` of this package.  There is no CPU fallback.
"""
from . import units
from ._capi import EngineError
from .system import (
    BerendsenThermostat,
    BornMayerHuggins,
    Buckingham,
    Engine,
    Ewald,
    Gaussian,
    Harmonic,
    LennardJones,
    Mie,
    MolecularDynamics,
    MonteCarlo,
    Morse,
    NullPotential,
    PairInteraction,
    PairRestriction,
    System,
    Translate,
    UnitCell,
    VelocityVerlet,
    Wolf,
)
from ._capi import (
    LG_TERM_ALL,
    LG_TERM_ANGLES,
    LG_TERM_BONDS,
    LG_TERM_COUL_KSPACE,
    LG_TERM_COUL_REAL,
    LG_TERM_COUL_SELF,
    LG_TERM_PAIRS,
    LG_TERM_TAIL,
)

__all__ = [
    "units", "EngineError", "BerendsenThermostat", "Buckingham", "Engine", "Ewald", "Harmonic",
    "LennardJones", "MolecularDynamics", "MonteCarlo", "Translate", "NullPotential", "PairInteraction", "PairRestriction",
    "System", "UnitCell", "VelocityVerlet", "Wolf",
    "LG_TERM_ALL", "LG_TERM_ANGLES", "LG_TERM_BONDS", "LG_TERM_COUL_KSPACE", "LG_TERM_COUL_REAL",
    "LG_TERM_COUL_SELF", "LG_TERM_PAIRS", "LG_TERM_TAIL",
]
