"""Triclinic cells on the CPU: the oracle's and the Python mirror's UnitCell
restatements pinned to the reference's own known answers
(lumol-core/src/sys/config/cells.rs tests `triclinic`, `lengths`,
`distances`, `wrap_vector`, `vector_image`, `fractional_cartesian`), and the
two restatements equal to each other bit for bit."""
import math

import numpy as np
import pytest

import lumol_gb300 as lg
import oracle


def _oracle_for(cell):
    s = lg.System(cell)
    s.add_particles(["Ar"], [[0.0, 0.0, 0.0]])
    s.set_pair_potential(("Ar", "Ar"), lg.PairInteraction(lg.LennardJones(1.0, 0.0), 0.5))
    return oracle.Oracle(s)


def _ulps(a, b):
    return abs(np.float64(a).view(np.int64) - np.float64(b).view(np.int64))


def test_constructor_and_volume_literals():
    """cells.rs `triclinic`: vect_a = (3, 0, 0), vect_b has no z, volume 55.410529."""
    c = lg.UnitCell.triclinic(3.0, 4.0, 5.0, 80.0, 90.0, 110.0)
    m = c.matrix()
    assert list(m[:, 0]) == [3.0, 0.0, 0.0]
    assert m[2, 1] == 0.0
    assert abs(c.volume() - 55.410529) <= 1e-6
    assert c.shape == "triclinic"
    orc = _oracle_for(c)
    lengths, volume = orc.cell_info()
    assert volume == c.volume()
    assert np.array_equal(orc.cell_matrix(), m)


def test_lengths_literals():
    """cells.rs `lengths` (assert_eq: exact)."""
    assert lg.UnitCell.ortho(3.0, 4.0, 5.0).lengths == (3.0, 4.0, 5.0)
    assert lg.UnitCell.triclinic(3.0, 4.0, 5.0, 90.0, 90.0, 90.0).lengths == (3.0, 4.0, 5.0)
    c = lg.UnitCell.triclinic(3.0, 4.0, 5.0, 90.0, 80.0, 100.0)
    expected = (2.908132319388713, 3.9373265973230853, 4.921658246653857)
    assert c.lengths == expected
    lengths, _ = _oracle_for(c).cell_info()
    assert tuple(lengths) == expected


def test_distance_wrap_and_image_literals():
    """cells.rs `distances` (exact), `wrap_vector` and `vector_image`
    (5 ulps) on the 90-degree triclinic cell."""
    c = lg.UnitCell.triclinic(3.0, 4.0, 5.0, 90.0, 90.0, 90.0)
    orc = _oracle_for(c)
    d = orc.cell_apply([1.0, 2.0, 6.0], "image")
    assert math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) == math.sqrt(6.0)
    for mode in ("wrap", "image"):
        v = orc.cell_apply([1.0, 1.5, 6.0], mode)
        for got, want in zip(v, (1.0, 1.5, 1.0)):
            assert _ulps(got, want) <= 5, (mode, v)
    w = c.wrap_vector([1.0, 1.5, 6.0])
    assert np.array_equal(np.array(w), orc.cell_apply([1.0, 1.5, 6.0], "wrap"))


def test_fractional_cartesian_round_trip():
    """cells.rs `fractional_cartesian` (1e-15)."""
    c = lg.UnitCell.triclinic(5.0, 6.0, 3.6, 90.0, 53.0, 77.0)
    orc = _oracle_for(c)
    for v in ([0.0, 10.0, 4.0], [-5.0, 12.0, 4.9]):
        back = orc.cell_apply(v, "roundtrip")
        assert np.abs(back - np.array(v)).max() <= 1e-15 * max(1.0, np.abs(v).max())
        assert np.array_equal(np.array(c.cartesian(c.fractional(v))), back)


def test_scaled_cell_keeps_the_shape():
    """UnitCell::scale_mut keeps the shape (cells.rs:201-207); the product is
    Matrix3's (a diagonal factor multiplies every entry)."""
    c = lg.UnitCell.triclinic(20.0, 21.0, 22.0, 80.0, 95.0, 105.0)
    s = c.scaled(1.01)
    assert s.shape == "triclinic"
    assert np.array_equal(s.matrix(), c.matrix() * 1.01)


def test_orthorhombic_cells_are_unchanged():
    """An orthorhombic cell keeps its lengths, volume and diagonal matrix."""
    c = lg.UnitCell.ortho(3.0, 4.0, 5.0)
    assert c.volume() == 60.0 and c.lengths == (3.0, 4.0, 5.0)
    assert np.array_equal(c.matrix(), np.diag([3.0, 4.0, 5.0]))
    with pytest.raises(ValueError):
        lg.UnitCell.triclinic(3.0, 0.0, -5.0, 90.0, 90.0, 90.0)
