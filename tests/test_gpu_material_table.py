"""Tabulated k(T) materials on the GPU against the oracle (set_material_table): piecewise k(T)
with an isotropic and an anisotropic table, a table with the thickness factor h**hexp, both
solvers, and the conductivity provider."""
import numpy as np
import pytest

from oracle import fem3d as O
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu

TOL_T = 1e-6


def _tabulated(seed, n):
    s = S.layered_c1(seed=seed, n=n)
    nm = s.k300.size
    s.hexp = np.zeros(nm)
    s.hexp[nm - 1] = 0.3  # the top material's table also scales with the layer thickness
    s.ktables = {
        0: (np.array([250.0, 320.0, 450.0, 900.0]), np.array([160.0, 120.0, 60.0, 30.0]), None),
        nm // 2: (np.array([280.0, 350.0, 700.0]), np.array([9.0, 6.0, 2.0]), np.array([4.0, 3.5, 1.0])),
        nm - 1: (np.array([300.0, 400.0]), np.array([30.0, 10.0]), np.array([30.0, 20.0])),
    }
    return s


@pytest.mark.parametrize("algorithm", ["gpu-mixed", "gpu-pcg"])
@pytest.mark.parametrize("n,order", [((16, 13, 20), "201"), ((19, 14, 17), "012")])
def test_tabulated_materials_match_oracle(algorithm, n, order):
    s = _tabulated(41, n)
    To, tot_o, rec = O.compute(O.from_structure(s, order=order))
    sv = TH.solver_for_structure(s, ordering=order, algorithm=algorithm)
    tot = sv.compute()
    T = sv._full_temperature()
    assert sv.stats["loops"] == len(rec)
    assert np.max(np.abs(T - To)) <= TOL_T
    assert abs(tot - tot_o) <= TOL_T


def test_tabulated_conductivity_provider():
    s = _tabulated(42, (12, 11, 15))
    p = O.from_structure(s, order="201")
    To, _, _ = O.compute(p)
    sv = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    sv.compute()
    kxy, kz = O.element_k(p, To)
    k = sv.outThermalConductivity()
    # linear tables: |dk|/k <= |slope| |dT| / k, far below 1e-8 at the temperature tolerance
    assert np.allclose(k[..., 0].ravel(), kxy, rtol=1e-8)
    assert np.allclose(k[..., 1].ravel(), kz, rtol=1e-8)
