"""lumol_gb300 -- a GB300 (sm_103a) engine for Lumol's force / energy /
virial / integration path, behind a C ABI (include/lumol_gb300.h).

The Python classes mirror lumol-core / lumol-sim (System, PairInteraction,
the pair potentials, Ewald, Wolf, the integrators, thermostats and controls,
MolecularDynamics, MonteCarlo); every computation runs in the CUDA library
`liblumol_gb300.so` of this package.  There is no CPU fallback.
"""
from . import units
from ._capi import EngineError
from .input import InputError, InteractionsInput, read_interactions
from .system import (
    AnisoBerendsenBarostat,
    BerendsenBarostat,
    BerendsenThermostat,
    BornMayerHuggins,
    Buckingham,
    CosineHarmonic,
    CSVRThermostat,
    Engine,
    Ewald,
    Gaussian,
    Harmonic,
    LeapFrog,
    LennardJones,
    Mie,
    MolecularDynamics,
    MonteCarlo,
    Morse,
    NullPotential,
    PairInteraction,
    PairRestriction,
    RemoveRotation,
    RemoveTranslation,
    RescaleThermostat,
    Resize,
    Rewrap,
    Rotate,
    System,
    TableComputation,
    Torsion,
    Translate,
    UnitCell,
    VelocityVerlet,
    Verlet,
    Wolf,
    md_params,
)
from ._capi import (
    LG_TERM_ALL,
    LG_TERM_ANGLES,
    LG_TERM_BONDS,
    LG_TERM_COUL_KSPACE,
    LG_TERM_COUL_REAL,
    LG_TERM_COUL_SELF,
    LG_TERM_DIHEDRALS,
    LG_TERM_PAIRS,
    LG_TERM_TAIL,
)

__all__ = [
    "units", "EngineError", "InputError", "InteractionsInput", "read_interactions", "BerendsenThermostat", "BornMayerHuggins", "Buckingham", "CSVRThermostat", "Engine",
    "Ewald", "Gaussian", "Harmonic", "LeapFrog", "LennardJones", "Mie", "MolecularDynamics", "MonteCarlo", "Morse",
    "Translate", "NullPotential", "PairInteraction", "PairRestriction", "RemoveRotation", "RemoveTranslation", "RescaleThermostat",
    "Rewrap", "Rotate", "System", "TableComputation", "Torsion", "CosineHarmonic", "UnitCell", "VelocityVerlet", "Verlet", "Wolf", "md_params",
    "LG_TERM_ALL", "LG_TERM_ANGLES", "LG_TERM_BONDS", "LG_TERM_COUL_KSPACE", "LG_TERM_COUL_REAL",
    "LG_TERM_COUL_SELF", "LG_TERM_DIHEDRALS", "LG_TERM_PAIRS", "LG_TERM_TAIL",
]
