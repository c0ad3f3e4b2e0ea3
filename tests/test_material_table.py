"""Tabulated k(T) materials (plgpu_fem3d_set_material_table) on the CPU: the oracle's table
evaluation, the Python material table's, and the oracle solve with a table that samples a
power law against the power law itself."""
import numpy as np

from oracle import fem3d as O
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH


def test_table_is_linear_between_points_and_constant_beyond():
    tab = (np.array([250.0, 300.0, 500.0]), np.array([10.0, 8.0, 4.0]), np.array([5.0, 6.0, 7.0]))
    T = np.array([100.0, 250.0, 275.0, 300.0, 400.0, 500.0, 900.0])
    kxy, kz = O.table_k(tab, T)
    assert np.allclose(kxy, [10.0, 10.0, 9.0, 8.0, 6.0, 4.0, 4.0], rtol=0, atol=1e-14)
    assert np.allclose(kz, [5.0, 5.0, 5.5, 6.0, 6.5, 7.0, 7.0], rtol=0, atol=1e-14)
    one = (np.array([300.0]), np.array([3.0]), None)
    assert np.all(O.table_k(one, T)[0] == 3.0)


def test_python_table_matches_oracle_and_hexp_applies():
    mt = TH.MaterialTable([1.0, 2.0], [1.0, 1.0], hexp=[0.0, 0.5])
    mt.tables = {1: (np.array([250.0, 600.0]), np.array([20.0, 5.0]), np.array([10.0, 2.5]))}
    m = np.array([0, 1, 1, 1])
    T = np.array([300.0, 260.0, 420.0, 700.0])
    h = np.array([1.0, 4.0, 0.25, 1.0])
    kxy, kz = mt.thermk(m, T, h)
    mats = O.Materials(mt.k300, mt.p, mt.kz_ratio, mt.hexp, mt.empty, mt.tables)
    okxy, okz = mats.thermk(m, T, h)
    assert np.allclose(kxy, okxy, rtol=1e-14) and np.allclose(kz, okz, rtol=1e-14)
    ref = O.table_k(mt.tables[1], T[1:])
    assert np.allclose(kxy[1:], ref[0] * h[1:] ** 0.5, rtol=1e-14)
    assert kxy[0] == 1.0 * (300.0 / 300.0) ** 1.0


def test_dense_table_of_a_power_law_reproduces_the_power_law_solve():
    s = S.layered_c0(seed=2, n=(9, 8, 12))
    To, tot_o, rec = O.compute(O.from_structure(s))
    grid = np.linspace(250.0, 900.0, 4001)
    s.ktables = {m: (grid, s.k300[m] * (300.0 / grid) ** s.p[m], None) for m in range(s.k300.size)}
    Tt, tot_t, rec_t = O.compute(O.from_structure(s))
    assert len(rec_t) == len(rec)
    assert np.max(np.abs(Tt - To)) < 1e-3  # linear interpolation error of the 0.16 K grid
