"""Shockley3D on the GPU against the CPU oracle (oracle/electr3d.py) and against
the closed-form answers of the reference's own test
(solvers/electrical/shockley/tests/shockley3d.py): a junction of area S between
two ideal conductors under 1 V carries 1e-9 S js (e^beta - 1) mA, dissipates that
current times 1 V, and has the capacitance eps0 eps S / d of a plate capacitor.

Tolerances: potentials within 1e-9 V of the oracle's Cholesky solution after the
same number of junction updates; current densities, heat densities and
conductivities within 1e-7 relative (of the field's maximum), 1e-5 in the diode
whose 1e9 S/m conductors turn a 5e-14 V rounding difference of the potential across a
0.5 um contact cell into 3e-6 kA/cm^2 of current (1e-5 of the 0.3 kA/cm^2 maximum); the closed-form current, heat and capacitance to the
decimal places the reference's test asks for (3, 3 and 2).

Nodes that only air elements touch (empty elements included) carry a potential
that 0.55e-14 S/m of air alone determines, 23 orders of magnitude below the
conductors; a solve that stops at the FP64 rounding floor of the whole system
leaves them within 1e-3 V of the direct solution (they carry no current).

The diode's loop stops on the largest change of the current density anywhere,
which in the 1e9 S/m conductors is rounding noise of about 1e-3 % for the Cholesky
oracle as for the GPU solver (one unit in the last place of the potential across
the 0.5 um contact cells); with the reference test's maxerr = 1e-3 % the loop ends
whenever the noise happens to dip below it (loop 140 for the oracle, 116-120 or
never for the GPU).  The closed-form checks therefore run a fixed 200 junction
updates, after which the junction itself has converged to 1e-7 %."""
import math

import numpy as np
import pytest

from oracle import electr3d as E
from oracle import fem3d as O
from plask_gb300 import electrical as EL
from plask_gb300 import structures as S

pytestmark = pytest.mark.gpu

EPS0_PF_UM = 8.854187817e-6  # pF/um


def _oracle_fields(p, V, conds):
    return E.currents(p, V, conds), E.heat(p, V, conds)


def _active_elements(s, exclude=True):
    return ~s.empty[s.mat] if exclude else np.ones(s.mat.shape, bool)


@pytest.mark.parametrize("algorithm", ["gpu-pcg", "gpu-mixed"])
def test_diode_closed_form(algorithm):
    s = S.shockley_diode()
    sv = EL.solver_for_structure(s, ordering="012", algorithm=algorithm)
    sv.maxerr = 0.0
    sv.compute(200)
    S_area = 1e6
    expected = 1e-9 * S_area * sv.js * (math.exp(sv.beta) - 1.0)
    I = sv.get_total_current()
    print(algorithm, "I", I, "expected", expected, "loops", sv.stats["total_loops"], "iters",
          sv.stats["inner_iterations"])
    assert round(I - expected, 3) == 0
    assert round(sv.get_total_heat() - expected * 1.0, 3) == 0
    C = sv.get_capacitance()
    assert round(C - EPS0_PF_UM * s.eps[1] * S_area / 0.02, 2) == 0


@pytest.mark.parametrize("empty_elements", ["exclude", "include"])
def test_diode_matches_oracle(empty_elements):
    s = S.shockley_diode()
    sv = EL.solver_for_structure(s, ordering="201", algorithm="gpu-pcg", empty_elements=empty_elements)
    loops = 12
    sv.compute(loops)
    p = E.from_structure(s, order="201", empty_elements=empty_elements)
    V, conds, toterr, rec = E.compute(p, loops=loops)
    Vg = sv._full_potential()
    solid = np.zeros(Vg.shape, bool)  # nodes of at least one non-empty element
    ne = ~s.empty[s.mat]
    for ck in (0, 1):
        for cj in (0, 1):
            for ci in (0, 1):
                solid[ck:ck + ne.shape[0], cj:cj + ne.shape[1], ci:ci + ne.shape[2]] |= ne
    air = np.isfinite(Vg) & ~solid
    print("max |dV|", np.max(np.abs(Vg[solid] - V[solid])), "air", np.max(np.abs(Vg[air] - V[air]), initial=0),
          "toterr", sv.err, toterr)
    assert np.max(np.abs(Vg[solid] - V[solid])) <= 1e-9
    assert np.max(np.abs(Vg[air] - V[air]), initial=0.0) <= 1e-3
    assert sv.stats["loops"] == len(rec)
    assert sv.err == pytest.approx(toterr, rel=1e-6, abs=1e-9)
    el = _active_elements(s, empty_elements == "exclude")
    j, h = _oracle_fields(p, V, conds)
    jg = sv.current_densities()
    assert np.all(np.isnan(jg[~el])) if empty_elements == "exclude" else np.all(np.isfinite(jg))
    sel = ~s.empty[s.mat]
    assert np.max(np.abs(jg[sel] - j[sel])) <= 1e-5 * np.max(np.abs(j[sel]))
    hg = sv.heat_densities()
    assert np.max(np.abs(hg - h)) <= 1e-5 * np.max(np.abs(h))
    cg = sv.conductivities()
    assert np.max(np.abs(cg[el] - conds[el])) <= 1e-7 * np.max(np.abs(conds[el]))
    assert sv.get_total_current() == pytest.approx(E.total_current(p, V, conds), rel=1e-7)
    assert sv.get_total_heat() == pytest.approx(E.total_heat(p, V, conds), rel=1e-7)


def test_diode_temperature_dependent_beta():
    """testComputationsTemp: beta(T) = ln(70 T) gives e^beta = 21000 at 300 K, 17500 at 250 K."""
    s = S.shockley_diode()
    sv = EL.solver_for_structure(s, ordering="012", algorithm="gpu-pcg")
    sv.beta = lambda T: math.log(T * 70)
    sv.maxerr = 0.0
    sv.compute(200)
    assert round(sv.get_total_current() - 1e-9 * 1e6 * sv.js * (21000 - 1), 3) == 0
    sv.inTemperature = 250.0
    sv.compute(200)
    assert round(sv.get_total_current() - 1e-9 * 1e6 * sv.js * (17500 - 1), 3) == 0


def test_diode_conductivity_before_compute():
    """testConductivity: material conductivity, (0, 5) S/m in the junction, NaN where excluded."""
    s = S.shockley_diode()
    sv = EL.solver_for_structure(s, ordering="012", algorithm="gpu-pcg")
    c = sv.conductivities()
    el = _active_elements(s)
    want = s.element_cond()
    want[s.junction > 0] = (0.0, 5.0)
    assert np.array_equal(c[el], want[el])
    assert np.all(np.isnan(c[~el]))


@pytest.mark.parametrize("convergence", ["fast", "stable"])
def test_layered_junction_matches_oracle(convergence):
    s = S.shockley_c4(seed=4001, n=(21, 19, 30), voltage=1.9)
    sv = EL.solver_for_structure(s, ordering="102", algorithm="gpu-mixed", convergence=convergence)
    loops = 5
    sv.compute(loops)
    p = E.from_structure(s, order="102", convergence=convergence)
    V, conds, toterr, rec = E.compute(p, loops=loops)
    Vg = sv._full_potential()
    print("max |dV|", np.max(np.abs(Vg - V)), "err", sv.err, toterr)
    assert np.max(np.abs(Vg - V)) <= 1e-9
    j, h = _oracle_fields(p, V, conds)
    jg = sv.current_densities()
    assert np.max(np.abs(jg - j)) <= 1e-7 * np.max(np.abs(j))
    hg = sv.heat_densities()
    assert np.max(np.abs(hg - h)) <= 1e-7 * np.max(np.abs(h))
    assert sv.err == pytest.approx(toterr, rel=1e-6)
    # the quarter structure: the factor 4 of the two symmetry planes
    assert sv.get_total_current() == pytest.approx(4 * E.total_current(p, V, conds), rel=1e-7)


def test_second_compute_continues_from_saved_junction():
    """compute(2) twice equals compute(4) once: the junction conductivities and the
    currents persist between calls (saveConductivity / loadConductivity)."""
    s = S.shockley_c4(seed=4002, n=(17, 17, 26), voltage=2.0)
    a = EL.solver_for_structure(s, ordering="012", algorithm="gpu-pcg")
    a.compute(2)
    a.compute(2)
    b = EL.solver_for_structure(s, ordering="012", algorithm="gpu-pcg")
    b.compute(4)
    assert np.max(np.abs(a._full_potential() - b._full_potential())) <= 1e-12
    assert a.stats["total_loops"] == b.stats["total_loops"] == 4


def test_thermoelectric_loop_matches_oracle():
    """ThermoElectric3D.compute against the same alternation on the CPU oracle:
    electrical compute(tfreq), Joule heat to the thermal problem, thermal compute(1)."""
    from plask_gb300 import thermal as TH

    s = S.shockley_c4(seed=4003, n=(19, 19, 28), voltage=2.1)
    te = EL.ThermoElectric3D()
    te.thermal = TH.solver_for_structure(s.thermal, ordering="012", algorithm="gpu-mixed")
    te.electrical = EL.solver_for_structure(s, ordering="012", algorithm="gpu-mixed")
    te.reconnect()
    verr, terr = te.compute()
    assert verr <= te.electrical.maxerr and terr <= te.thermal.maxerr

    p = E.from_structure(s, order="012")
    tp = O.from_structure(s.thermal, order="012")
    state, T, rounds = {}, None, []
    ve, tt = 2 * s.maxerr, 2 * tp.maxerr
    while tt > tp.maxerr or ve > s.maxerr:
        V, conds, ve, _ = E.compute(p, loops=te.tfreq, state=state)
        tp.heat = E.heat(p, V, conds)
        T, tt, _ = O.compute(tp, loops=1, T=T)
        rounds.append((ve, tt))
    print("gpu rounds", te.history, "oracle rounds", rounds)
    assert len(rounds) == len(te.history)
    Tg = te.thermal._full_temperature()
    assert np.max(np.abs(Tg - T)) <= 1e-6
    Vg = te.electrical._full_potential()
    assert np.max(np.abs(Vg - V)) <= 1e-9
