"""The allocation-free Ewald k-space entry point, lg_ewald_kspace_noalloc.

It serves callers that cannot call cudaMalloc: code running inside a host
framework whose pool allocator owns the device memory, and per-step or
per-move loops where an allocation would synchronise the device.  These tests
call it through the C ABI on device buffers the test owns, two calls in a row,
and check each result against lg_compute(LG_TERM_COUL_KSPACE) of the regular
engine and against the oracle's Ewald k-space terms, at the parity tolerance
of the other GPU tests (1e-10).  They also check that the calls leave the
device's free memory unchanged, that a call on a side stream gives the same
result, and the edge cases kmax = 1 (no k-vector) and n = 0.  The file name
makes pytest collect it after every other test file.
"""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
from lumol_gb300 import _capi as C
from lumol_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _engine(system):
    return system.compute(lg.LG_TERM_COUL_KSPACE)


def _oracle(system):
    orc = oracle.Oracle(system)
    t = oracle.TERM_COUL_KSPACE
    return orc.forces(t), orc.energy(t), orc.virial(t)


class _Buffers:
    """Device inputs and outputs of one system, owned by the test."""

    def __init__(self, system):
        import torch
        n = system.size
        self.n = n
        self.pos = torch.tensor(np.ascontiguousarray(system.positions).reshape(n, 3), dtype=torch.float64,
                                device="cuda")
        self.charges = torch.tensor(np.asarray(system.charges, dtype=np.float64), device="cuda")
        self.forces = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        self.energy = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.virial = torch.zeros(9, dtype=torch.float64, device="cuda")
        self.cell = (ctypes.c_double * 3)(*system.cell.lengths)
        self.alpha = system.coulomb.alpha
        self.kmax = system.coulomb.kmax

    def call(self, stream=None):
        """One call; the forces are accumulated into a zeroed buffer.  Also
        returns the device's free memory just before and just after the call
        (the test's own buffer preparation is outside that window)."""
        import torch
        self.forces.zero_()
        self.energy.fill_(np.nan)
        self.virial.fill_(np.nan)
        torch.cuda.synchronize()
        handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
        free_before, _ = torch.cuda.mem_get_info()
        rc = C.load().lg_ewald_kspace_noalloc(self.pos.data_ptr(), self.charges.data_ptr(), self.n, self.cell,
                                              self.alpha, self.kmax, self.forces.data_ptr(),
                                              self.energy.data_ptr(), self.virial.data_ptr(), handle)
        C.check(rc)
        torch.cuda.synchronize()
        free_after, _ = torch.cuda.mem_get_info()
        self.free = (free_before, free_after)
        return (self.forces.cpu().numpy(), float(self.energy.item()), self.virial.cpu().numpy().reshape(3, 3))


def _assert_close(got, ref, what):
    f, e, w = got
    fo, eo, wo = ref
    wo = np.asarray(wo).reshape(3, 3)
    assert abs(e - eo) <= TOL * abs(eo), (what, e, eo)
    assert np.abs(w - wo).max() <= TOL * np.abs(wo).max(), (what, w, wo)
    err = np.sqrt(np.mean((f - fo) ** 2)) / np.sqrt(np.mean(fo ** 2))
    assert err <= TOL, (what, err)


@pytest.mark.parametrize("make", [
    lambda: workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5),
    lambda: workloads.nacl_crystal(),
    lambda: workloads.water_box(n_side=7, length=21.76),
], ids=["nacl216_kmax5", "nacl1000_kmax7", "water343_kmax8"])
def test_noalloc_matches_engine_and_oracle_on_two_calls(make):
    system = make()
    ref_engine = _engine(system)
    ref_oracle = _oracle(system)
    buf = _Buffers(system)
    for call in range(2):
        got = buf.call()
        _assert_close(got, ref_engine, f"call {call} vs engine")
        _assert_close(got, ref_oracle, f"call {call} vs oracle")


def test_noalloc_allocates_nothing_and_honours_the_stream():
    import torch
    system = workloads.nacl_crystal()
    ref = _oracle(system)
    buf = _Buffers(system)
    side = torch.cuda.Stream()
    buf.call()  # warm-up on both streams: module loading, the scratch address, torch's own kernels
    with torch.cuda.stream(side):
        buf.call(side)
    with torch.cuda.stream(side):
        got_side = buf.call(side)
    assert buf.free[1] == buf.free[0], ("side stream", buf.free)
    got_default = buf.call()
    assert buf.free[1] == buf.free[0], ("default stream", buf.free)
    _assert_close(got_side, ref, "side stream")
    _assert_close(got_default, ref, "default stream after the side stream")


def test_noalloc_edge_cases_kmax1_and_empty():
    # kmax = 1: Ewald::prepare's loops run over 1..kmax, so there is no k-vector
    # and every k-space term is zero (ewald.rs:146-182)
    system = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=1)
    buf = _Buffers(system)
    for _ in range(2):
        f, e, w = buf.call()
        assert e == 0.0 and np.all(w == 0.0) and np.all(f == 0.0)
    assert _oracle(system)[1] == 0.0
    # n = 0: energy and virial are written (zero), no forces are touched
    lib = C.load()
    import torch
    energy = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
    virial = torch.full((9,), np.nan, dtype=torch.float64, device="cuda")
    cell = (ctypes.c_double * 3)(20.0, 20.0, 20.0)
    for _ in range(2):
        C.check(lib.lg_ewald_kspace_noalloc(None, None, 0, cell, 0.3, 5, None, energy.data_ptr(),
                                            virial.data_ptr(), None))
        torch.cuda.synchronize()
        assert float(energy.item()) == 0.0 and torch.all(virial == 0.0)


def test_noalloc_rejects_sizes_beyond_its_limit():
    lib = C.load()
    cell = (ctypes.c_double * 3)(30.0, 30.0, 30.0)
    rc = lib.lg_ewald_kspace_noalloc(None, None, 4097, cell, 0.3, 5, None, None, None, None)
    assert rc == C.LG_ERR_ARGUMENT
    assert b"4096" in lib.lg_last_error(None)
    rc = lib.lg_ewald_kspace_noalloc(None, None, 10, cell, 0.3, 9, None, None, None, None)
    assert rc == C.LG_ERR_ARGUMENT
    assert b"kmax" in lib.lg_last_error(None)
