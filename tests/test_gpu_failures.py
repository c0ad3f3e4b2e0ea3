"""Failure detection through the status word and the C ABI's error codes, with inputs that
produce each status (nothing faults or hangs the GPU): an iteration cap under the three
`noconv` behaviours of the reference (iterative_matrix.hpp:299-315), a non-finite heat
source, and arguments the library rejects."""
import logging

import numpy as np
import pytest

from plask_gb300 import _native
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu


def _solver(**kw):
    s = S.layered_c0(seed=3, n=(12, 12, 16))
    sv = TH.solver_for_structure(s, algorithm="iterative", **kw)
    return s, sv


def test_iteration_cap_with_noconv_error_raises():
    _, sv = _solver()
    sv.iterative.maxit = 5
    sv.iterative.noconv = "error"
    with pytest.raises(TH.ComputationError) as ei:
        sv.compute(1)
    assert ei.value.code == _native.ERR_NOCONV
    assert "failed to converge" in str(ei.value)


def test_iteration_cap_with_noconv_warning_keeps_looping(caplog):
    _, sv = _solver()
    sv.iterative.maxit = 5
    sv.iterative.noconv = "warning"
    with caplog.at_level(logging.WARNING, logger="plask_gb300.thermal"):
        sv.compute(2)
    # an unconverged solve keeps the outer loop going until the loop limit
    assert sv.stats["loops"] == 2
    assert not sv.iterative.converged
    assert any("Failed to converge" in r.getMessage() for r in caplog.records if r.levelno == logging.WARNING)


def test_iteration_cap_with_noconv_continue_is_silent(caplog):
    _, sv = _solver()
    sv.iterative.maxit = 5
    sv.iterative.noconv = "continue"
    with caplog.at_level(logging.WARNING, logger="plask_gb300.thermal"):
        sv.compute(2)
    assert not sv.iterative.converged
    assert not [r for r in caplog.records if r.levelno >= logging.WARNING]


def test_non_finite_heat_is_reported():
    s, sv = _solver()
    heat = np.array(s.heat, dtype=np.float64)
    heat.flat[heat.size // 2] = np.nan
    sv.inHeat = heat
    with pytest.raises(TH.ComputationError) as ei:
        sv.compute(1)
    assert ei.value.code == _native.ERR_NONFINITE


def test_bad_arguments_are_rejected():
    ax = np.linspace(0.0, 1.0, 4)
    with pytest.raises(_native.BadInput):
        _native.Fem3D((ax, np.array([0.0, 1.0, 0.5]), ax))  # axis not increasing
    fem = _native.Fem3D((ax, ax, ax))
    with pytest.raises(_native.BadInput):
        fem.set_materials(np.array([-1.0]), np.array([0.0]))  # negative conductivity
    fem.set_materials(np.array([10.0]), np.array([0.0]))
    with pytest.raises(_native.BadInput):
        fem.set_elements(np.full(27, 3, np.int32))  # material id out of range
    with pytest.raises(_native.BadInput):
        fem.set_solver("iterative", noconv="error", empty_elements="default")  # accepted names pass...
        fem.set_dynamic(np.ones(1), np.ones(1), timestep=-1.0)  # ...a negative timestep does not
    with pytest.raises(_native.NativeError):
        fem.compute(0)  # elements never set
