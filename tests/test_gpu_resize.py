"""NPT Monte Carlo on the GPU: EnergyCache::move_all_molecules_cost
(lumol-core/src/sys/cache.rs:238-292) for Resize moves
(lumol-sim/src/mc/moves/resize.rs:63-124), against the oracle's restatement
(1e-10 of the energy), with accepted and rejected moves in sequence."""
import ctypes

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle
import systems
from lumol_gb300 import _capi as C
from lumol_gb300 import units, workloads
from lumol_gb300.system import _ortho_inverse

pytestmark = pytest.mark.gpu


def _resized(s, L, pos, factor):
    """The cell and positions Resize::prepare makes for a volume factor."""
    L_new = np.asarray(L) * np.cbrt(factor)
    inv = _ortho_inverse(L)
    m = s.masses
    out = pos.copy()
    for mol in range(int(s.molecules[-1]) + 1):
        lo, hi = s.molecule_range(mol)
        com = (m[lo:hi, None] * pos[lo:hi]).sum(axis=0) / m[lo:hi].sum()
        out[lo:hi] = pos[lo:hi] + (L_new * (inv * com) - com)
    return L_new, out


def _cost(eng, L_new, pos):
    c = ctypes.c_double()
    eng.call("lg_mc_move_all_molecules_cost", 0, C.dptr(np.diag(L_new).ravel().copy()),
             C.dptr(np.ascontiguousarray(pos)), ctypes.byref(c))
    return c.value


@pytest.mark.parametrize("make", [
    lambda: workloads.lj_replica(400, 0.5, 150.0, seed=3),
    lambda: systems.chains(27, 24.0, 3, lg.PairRestriction.INTER_MOLECULAR),
], ids=["lj_fluid", "chains"])
def test_resize_costs_follow_the_oracle(make):
    s = make()
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = s.mc_init()
    scale = abs(e0)
    assert abs(e0 - orc.cache_energy()) <= 1e-10 * scale
    eng = s.engine()
    L = np.array(s.cell.lengths)
    pos = s.positions.copy()
    for k, (factor, accept) in enumerate([(1.03, True), (0.97, False), (0.985, True), (1.01, False),
                                          (1.005, True)]):
        L_new, newpos = _resized(s, L, pos, factor)
        cost = _cost(eng, L_new, newpos)
        ref = orc.move_all_molecules_cost(L_new, newpos)
        assert abs(cost - ref) <= 1e-10 * scale, (k, cost, ref)
        if accept:
            energy = ctypes.c_double()
            eng.call("lg_mc_update", 0, None, ctypes.byref(energy))
            orc.cache_update()
            assert abs(energy.value - orc.cache_energy()) <= 1e-10 * scale
            L, pos = L_new, newpos
        else:
            eng.call("lg_mc_restore", 0)
            orc.cache_restore()
    # a single-molecule move after the resizes sees the accepted configuration
    lo, hi = s.molecule_range(5)
    moved = pos[lo:hi] + np.array([0.2, -0.1, 0.15])
    c = ctypes.c_double()
    eng.call("lg_mc_move_molecule_cost", 0, 5, C.dptr(np.ascontiguousarray(moved)), ctypes.byref(c))
    orc.set_positions(pos)
    assert abs(c.value - orc.move_molecule_cost(5, moved)) <= 1e-10 * scale
    cell = np.zeros(9)
    eng.call("lg_get_cell", 0, C.dptr(cell))
    assert np.array_equal(cell[[0, 4, 8]], L)


def test_resize_with_ewald_follows_the_oracle():
    s = workloads.nacl_crystal(cells=3, cutoff=8.0, kmax=5)
    orc = oracle.Oracle(s)
    orc.cache_init()
    e0 = s.mc_init()
    eng = s.engine()
    L_new, newpos = _resized(s, np.array(s.cell.lengths), s.positions.copy(), 1.02)
    cost = _cost(eng, L_new, newpos)
    assert abs(cost - orc.move_all_molecules_cost(L_new, newpos)) <= 1e-10 * abs(e0)


def test_npt_monte_carlo_keeps_its_cache():
    """Translate + Resize moves (MonteCarlo::add with frequencies) at a pressure
    away from the starting one: the volume moves, and after 300 moves the
    cached energy equals a fresh evaluation of the final configuration."""
    s = workloads.lj_replica(300, 0.4, 120.0, seed=9)
    V0 = s.volume()
    mc = lg.MonteCarlo(120.0, [(lg.Translate(0.4), 0.8), (lg.Resize(units.from_(500.0, "bar"), 60.0), 0.2)],
                       seed=2)
    mc.setup(s)
    for _ in range(300):
        mc.propagate(s)
    assert mc.accepted > 0 and s.volume() != V0
    fresh = s.potential_energy()
    assert abs(mc.energy - fresh) <= 1e-9 * abs(fresh)


def test_resize_below_twice_the_cutoff_fails_like_the_reference():
    s = workloads.lj_replica(300, 0.4, 120.0, seed=9)
    s.mc_init()
    L = np.array(s.cell.lengths)
    L_new, newpos = _resized(s, L, s.positions.copy(), ((2 * 2.5 * 3.405) / L[0]) ** 3 * 0.99)
    with pytest.raises(lg.EngineError, match="Tried to decrease the cell size in Monte Carlo Resize move"):
        _cost(s.engine(), L_new, newpos)
