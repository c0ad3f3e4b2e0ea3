"""CPU tests of the Shockley3D oracle (oracle/electr3d.py, a restatement of
solvers/electrical/shockley/electr3d.cpp) against the closed-form answers of the
reference's own test (solvers/electrical/shockley/tests/shockley3d.py:62-91): a p-n
junction of area S = 1e6 um^2 between ideal conductors carries the current
1e-9 S js (e^beta - 1) mA and dissipates that times 1 V, and its capacitance is
eps0 eps S / 0.02 um.  The loop runs a fixed 200 junction updates (the test's stopping
value is at the rounding noise of the contacts' currents)."""
import math

import numpy as np
import pytest

from oracle import electr3d as E
from plask_gb300 import structures as S

EPS0_PF_UM = 8.854187817e-6  # pF/um
AREA = 1e6  # um^2


@pytest.fixture(scope="module")
def diode():
    s = S.shockley_diode()
    p = E.from_structure(s, order="012", maxerr=0.0)
    V, conds, _, rec = E.compute(p, loops=200)
    return s, p, V, conds, rec


def test_current_and_heat_of_the_reference_diode(diode):
    s, p, V, conds, rec = diode
    assert len(rec) == 200
    expected = 1e-9 * AREA * s.js[0] * (math.exp(s.beta[0]) - 1.0)  # mA
    current = E.total_current(p, V, conds)
    assert round(current - expected, 3) == 0
    assert round(E.total_heat(p, V, conds) - expected * 1.0, 3) == 0


def test_capacitance_of_the_reference_diode(diode):
    s, p, V, conds, _ = diode
    eps_elem = s.eps[s.mat]
    energy = E.total_energy(p, V, eps_elem)  # J
    u = 1.0  # V between the contacts
    capacitance = 2.0 * energy / (u * u) * 1e12  # pF
    assert round(capacitance - EPS0_PF_UM * s.eps[1] * AREA / 0.02, 2) == 0

