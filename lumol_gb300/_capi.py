"""ctypes binding of the C ABI declared in include/lumol_gb300.h.

The shared library is loaded from this package directory.  There is no CPU
fallback: a missing library, or a machine without a CUDA device, raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblumol_gb300.so")

LG_OK = 0
LG_ERR_ARGUMENT = 1
LG_ERR_CUDA = 2
LG_ERR_STATE = 3
LG_ERR_CAPACITY = 4
LG_ERR_NONFINITE = 5
LG_ERR_NO_DEVICE = 6

LG_PAIR_ABSENT, LG_PAIR_NULL, LG_PAIR_LJ, LG_PAIR_BUCKINGHAM, LG_PAIR_HARMONIC = range(5)
LG_PAIR_BMH, LG_PAIR_MORSE, LG_PAIR_GAUSSIAN, LG_PAIR_MIE = range(5, 9)
LG_COULOMB_NONE, LG_COULOMB_EWALD, LG_COULOMB_WOLF = range(3)
LG_PRECISION_FP64, LG_PRECISION_MIXED = 0, 1
LG_OPT_NO_PERSISTENT = 1
LG_OPT_STAGING = 2
LG_OPT_CLUSTER_SHIFT = 4

LG_TERM_PAIRS = 1
LG_TERM_TAIL = 2
LG_TERM_BONDS = 4
LG_TERM_ANGLES = 8
LG_TERM_COUL_REAL = 16
LG_TERM_COUL_SELF = 32
LG_TERM_COUL_KSPACE = 64
LG_TERM_DIHEDRALS = 128
LG_TERM_ALL = 255
LG_BONDED_COSINE_HARMONIC, LG_BONDED_TORSION = 10, 11

LG_SYNC_DOWNLOAD = 1
LG_SYNC_TRUST_HOST = 2
LG_SYS_NONFINITE = 1

LG_WANT_FORCES = 1
LG_WANT_ENERGY = 2
LG_WANT_VIRIAL = 4


class LgPair(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("shifted", ctypes.c_int32),
        ("restriction", ctypes.c_int32),
        ("tail", ctypes.c_int32),
        ("p0", ctypes.c_double),
        ("p1", ctypes.c_double),
        ("p2", ctypes.c_double),
        ("cutoff", ctypes.c_double),
        ("scale14", ctypes.c_double),
        ("p3", ctypes.c_double),
        ("p4", ctypes.c_double),
        ("table_size", ctypes.c_int32),
        ("table_pad", ctypes.c_int32),
        ("table_max", ctypes.c_double),
    ]


class LgBonded(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("n", ctypes.c_int32), ("k", ctypes.c_double), ("x0", ctypes.c_double),
                ("a", ctypes.c_double)]


class LgCoulomb(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("restriction", ctypes.c_int32),
        ("kmax", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("cutoff", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("scale14", ctypes.c_double),
    ]


class LgOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("precision", ctypes.c_int32), ("skin", ctypes.c_double),
                ("threads_per_atom", ctypes.c_int32), ("flags", ctypes.c_int32)]


LG_INTEGRATOR_VELOCITY_VERLET, LG_INTEGRATOR_VERLET, LG_INTEGRATOR_LEAP_FROG = 0, 1, 2
LG_THERMOSTAT_NONE, LG_THERMOSTAT_BERENDSEN, LG_THERMOSTAT_RESCALE, LG_THERMOSTAT_CSVR = 0, 1, 2, 3
LG_CONTROL_REMOVE_TRANSLATION, LG_CONTROL_REWRAP, LG_CONTROL_REMOVE_ROTATION = 1, 2, 4
LG_BAROSTAT_NONE, LG_BAROSTAT_BERENDSEN, LG_BAROSTAT_ANISO_BERENDSEN = 0, 1, 2
LG_CELL_ORTHORHOMBIC, LG_CELL_TRICLINIC = 0, 1


class LgMdParams(ctypes.Structure):
    _fields_ = [("integrator", ctypes.c_int32), ("thermostat", ctypes.c_int32), ("timestep", ctypes.c_double),
                ("temperature", ctypes.c_double), ("tau", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("controls", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


# name -> (restype, argtypes)
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
SIGNATURES = {
    "lg_version": (ctypes.c_int, []),
    "lg_last_error": (ctypes.c_char_p, [_P]),
    "lg_create": (ctypes.c_int, [ctypes.POINTER(LgOptions), ctypes.c_int32, ctypes.POINTER(_P)]),
    "lg_destroy": (None, [_P]),
    "lg_set_cell": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "lg_set_cell_ex": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_int32]),
    "lg_set_particles": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, _I32, _D, _D, _I32]),
    "lg_set_bonds": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, _I32, ctypes.POINTER(LgBonded)]),
    "lg_set_angles": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, _I32, ctypes.POINTER(LgBonded)]),
    "lg_set_dihedrals": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, _I32, ctypes.POINTER(LgBonded)]),
    "lg_set_pairs": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(LgPair)]),
    "lg_set_coulomb": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(LgCoulomb)]),
    "lg_compute": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_uint32, ctypes.c_uint32, _D, _D, _D]),
    "lg_molecular_virial": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_uint32, _D]),
    "lg_compute_device": (ctypes.c_int, [_P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, _P, _P, _P]),
    "lg_pairset": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_int32, _I32, ctypes.c_int64, _I64]),
    "lg_md_setup": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "lg_md_setup_ex": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(LgMdParams)]),
    "lg_list_cells": (ctypes.c_int, [_P, ctypes.c_int32, _I32, _I32]),
    "lg_md_set_barostat": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double]),
    "lg_get_cell": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "lg_md_set_aniso_barostat": (ctypes.c_int, [_P, ctypes.c_int32, _D, ctypes.c_double]),
    "lg_cell_info": (ctypes.c_int, [_P, ctypes.c_int32, _I32, _D, _D]),
    "lg_md_set_state": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D]),
    "lg_md_get_state": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D]),
    "lg_md_set_state_all": (ctypes.c_int, [_P, _D, _D, _D]),
    "lg_md_get_state_all": (ctypes.c_int, [_P, _D, _D, _D]),
    "lg_md_run": (ctypes.c_int, [_P, ctypes.c_int64]),
    "lg_md_set_state_ex": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D, _D]),
    "lg_md_get_state_ex": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D, _D]),
    "lg_add_systems": (ctypes.c_int, [_P, ctypes.c_int32]),
    "lg_remove_system": (ctypes.c_int, [_P, ctypes.c_int32]),
    "lg_md_integrate": (ctypes.c_int, [_P, _D, _D, ctypes.c_int64]),
    "lg_md_propagate": (ctypes.c_int, [_P, _D, _D, ctypes.c_int64, ctypes.c_uint32]),
    "lg_system_status": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int32]),
    "lg_mc_init": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D]),
    "lg_mc_move_molecule_cost": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int64, _D, _D]),
    "lg_mc_update": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D]),
    "lg_mc_move_all_molecules_cost": (ctypes.c_int, [_P, ctypes.c_int32, _D, _D, _D]),
    "lg_mc_restore": (ctypes.c_int, [_P, ctypes.c_int32]),
    "lg_mc_setup": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]),
    "lg_mc_setup_ex": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_uint64]),
    "lg_mc_run": (ctypes.c_int, [_P, ctypes.c_int64]),
    "lg_mc_stats": (ctypes.c_int, [_P, ctypes.c_int32, _D, _I64, _I64]),
    "lg_get_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "lg_kernel_times": (ctypes.c_int, [_P, ctypes.c_int32, _D]),
    "lg_launch_count": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "lg_md_plan": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "lg_fma_peak": (ctypes.c_int, [ctypes.c_int32, _D]),
    "lg_test_stale_cell_counts": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "lg_ewald_kspace_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_int64, _D, ctypes.c_double, ctypes.c_int32,
                                               _P, _P, _P, _P]),
}

LG_KT_NAMES = ["nlist", "pair", "bonded", "eikr", "rho", "field", "vv", "step"]

_lib = None


class EngineError(RuntimeError):
    """A failure reported by the engine (the reference panics in these cases)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[lumol_gb300 error {code}] {message}")
        self.code = code


def load() -> ctypes.CDLL:
    """Loads the engine library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m lumol_gb300.build` "
                "(the engine has no CPU fallback)"
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code: int, handle=None) -> None:
    if code != LG_OK:
        msg = load().lg_last_error(handle)
        raise EngineError(code, msg.decode() if msg else "unknown error")


def dptr(array) -> ctypes.POINTER(ctypes.c_double):
    return array.ctypes.data_as(_D)


def iptr(array) -> ctypes.POINTER(ctypes.c_int32):
    return array.ctypes.data_as(_I32)
