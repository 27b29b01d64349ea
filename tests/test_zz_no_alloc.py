"""The allocation-free Ewald k-space entry point, lg_ewald_kspace_noalloc.

It serves callers that cannot call cudaMalloc (a host framework whose pool
allocator owns the device memory, or a per-step / per-move loop where an
allocation would synchronise the device).  This test calls it through the C
ABI on device buffers the test owns, twice in a row, and checks each result
against lg_compute(LG_TERM_COUL_KSPACE) of the regular engine at the parity
tolerance of the other GPU tests (1e-10).  The file name makes pytest collect
it after every other test file.
"""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
from lumol_gb300 import _capi as C
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _reference(system):
    return system.compute(lg.LG_TERM_COUL_KSPACE)


def _noalloc(system):
    import torch
    n = system.size
    pos = torch.tensor(np.ascontiguousarray(system.positions), dtype=torch.float64, device="cuda")
    charges = torch.tensor(system.charges, dtype=torch.float64, device="cuda")
    forces = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    energy = torch.zeros(1, dtype=torch.float64, device="cuda")
    virial = torch.zeros(9, dtype=torch.float64, device="cuda")
    cell = (ctypes.c_double * 3)(*system.cell.lengths)
    torch.cuda.synchronize()
    rc = C.load().lg_ewald_kspace_noalloc(pos.data_ptr(), charges.data_ptr(), n, cell, system.coulomb.alpha,
                                          system.coulomb.kmax, forces.data_ptr(), energy.data_ptr(),
                                          virial.data_ptr(), None)
    C.check(rc)
    torch.cuda.synchronize()
    return forces.cpu().numpy(), float(energy.item()), virial.cpu().numpy().reshape(3, 3)


def _assert_close(got, ref):
    f, e, w = got
    fo, eo, wo = ref
    assert abs(e - eo) <= TOL * abs(eo), (e, eo)
    assert np.abs(w - wo).max() <= TOL * np.abs(wo).max(), (w, wo)
    err = np.sqrt(np.mean((f - fo) ** 2)) / np.sqrt(np.mean(fo ** 2))
    assert err <= TOL, err


@pytest.mark.parametrize("make", [
    lambda: workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5),
    lambda: workloads.nacl_crystal(),
    lambda: workloads.water_box(n_side=7, length=21.76),
])
def test_noalloc_matches_engine_on_two_calls(make):
    system = make()
    ref = _reference(system)
    first = _noalloc(system)
    second = _noalloc(system)
    _assert_close(first, ref)
    _assert_close(second, ref)


def test_noalloc_rejects_sizes_beyond_its_limit():
    lib = C.load()
    cell = (ctypes.c_double * 3)(30.0, 30.0, 30.0)
    rc = lib.lg_ewald_kspace_noalloc(None, None, 4097, cell, 0.3, 5, None, None, None, None)
    assert rc == C.LG_ERR_ARGUMENT
    assert b"4096" in lib.lg_last_error(None)
    rc = lib.lg_ewald_kspace_noalloc(None, None, 10, cell, 0.3, 9, None, None, None, None)
    assert rc == C.LG_ERR_ARGUMENT
    assert b"kmax" in lib.lg_last_error(None)
