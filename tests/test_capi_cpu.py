"""CPU checks of the C ABI: the library loads, exports every function that
include/lumol_gb300.h declares, and fails loudly (no CPU fallback) when no
GPU is visible."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "lumol_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    from lumol_gb300 import _capi
    lib = _capi.load()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lg_[a-z0-9_]+)", out))
    assert set(names) <= exported


def test_python_binding_covers_the_header():
    from lumol_gb300 import _capi
    assert set(declared_functions()) == set(_capi.SIGNATURES)


def test_version():
    from lumol_gb300 import _capi
    assert _capi.load().lg_version() == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_loudly():
    import lumol_gb300 as lg
    with pytest.raises(lg.EngineError) as err:
        lg.Engine(1)
    assert err.value.code == 6  # LG_ERR_NO_DEVICE
    assert "no CPU fallback" in str(err.value)


def test_host_checks_mirror_reference_panics():
    import lumol_gb300 as lg
    with pytest.raises(ValueError, match="kmax can not be 0"):
        lg.Ewald(8.0, 0)
    with pytest.raises(ValueError, match="negative"):
        lg.Ewald(-8.0, 10)
    with pytest.raises(ValueError, match="Wolf"):
        lg.Wolf(-1.0)
    with pytest.raises(ValueError, match="half of the smallest cell"):
        s = lg.System(lg.UnitCell.cubic(10.0))
        s.set_pair_potential(("A", "A"), lg.PairInteraction(lg.LennardJones(1.0, 1.0), 5.5))
    with pytest.raises(ValueError, match="berendsen"):
        lg.BerendsenThermostat(300.0, 0.5)
    # functions.rs:774-777 and 803-806 (should_panic tests)
    with pytest.raises(ValueError, match="positive in Gaussian"):
        lg.Gaussian(8.0, -2.0)
    with pytest.raises(ValueError, match="larger than the attractive exponent"):
        lg.Mie(2.0, 0.8, 6.0, 12.0)
    # thermostats.rs:228-259 (should_panic tests)
    with pytest.raises(ValueError, match="positive in thermostats"):
        lg.RescaleThermostat(-56.0)
    with pytest.raises(ValueError, match="positive in thermostats"):
        lg.CSVRThermostat(-56.0, 1000.0)
    with pytest.raises(ValueError, match="larger than 1 in CSVR"):
        lg.CSVRThermostat(56.0, 0.3)
    with pytest.raises(ValueError, match="larger than 1 in berendsen"):
        lg.BerendsenThermostat(56.0, -2.0)


def test_units_match_reference_conversions():
    """lumol-core/src/units.rs:455-499, for the expressions without parentheses."""
    from lumol_gb300 import units
    assert units.from_(1.0, "bohr/fs") == 0.52917720859
    assert units.from_(1.0, "kJ/mol/deg^2") == 0.3282806352310398
    assert abs(units.from_(1.0, "kcal/mol/A^2") - 4.184e-4) <= 1e-9
    assert units.to(25.0, "m") == 2.5e-9
    assert units.to(25.0, "bar") == 4.1513469550000005e9
    assert units.to(25.0, "kJ/mol") == 249999.99982494753
    assert units.from_(10.0, "nm") == 100.0
