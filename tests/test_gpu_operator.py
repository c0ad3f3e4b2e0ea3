"""The matrix-free operator against the oracle's assembled system matrix (FemMatrix::mult).

A x is compared with the oracle's setMatrix + applyBC matrix for random x, at
the initial temperature and after one outer loop (temperature-dependent k),
for isotropic and anisotropic materials, several mesh orders, and convective,
heat-flux and radiative boundaries."""
import numpy as np
import pytest

from oracle import fem3d as O
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu


def _structure(kind, seed):
    if kind == "iso":
        s = S.layered_c0(seed=seed, n=(13, 11, 17))
    else:
        s = S.layered_c1(seed=seed, n=(35, 33, 21))  # wider than one 30-column tile and several row tiles
    s.heatflux = [("left", -2e4)]
    s.radiation = [("front", 0.7, 310.0)]
    return s


@pytest.mark.parametrize("order", ["201", "012", "120"])
@pytest.mark.parametrize("kind", ["iso", "aniso"])
@pytest.mark.parametrize("after_loop", [False, True])
def test_mult_matches_oracle_matrix(kind, order, after_loop):
    s = _structure(kind, 21)
    sv = TH.solver_for_structure(s, ordering=order, algorithm="gpu-mixed")
    sv.initialize()
    if after_loop:
        sv.compute(1)
    T = sv._full_temperature()
    p = O.from_structure(s, order=order)
    A, F, node_id, n = O.assemble(p, T)
    is_d, vf, vl = O.dirichlet_values(p, node_id, n)
    A2, _ = O.apply_dirichlet(A, F, is_d, vf, vl)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n)
    ref = A2 @ x
    y64 = sv._fem.mult(x, 64)
    y32 = sv._fem.mult(x, 32)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(y64 - ref)) <= 1e-12 * scale
    assert np.max(np.abs(y32 - ref)) <= 2e-5 * scale


# Meshes the TMA-staged CG kernel takes: one to four warps along x (64, 128, 192 and 248
# columns: one or two copy regions), partial row tiles, several z-chunks, convective top
# faces (surface rows in one plane) and side conditions (surface rows in every plane); and,
# with PLGPU_TMA_ALWAYS=1, widths it fills only partly (36, 40, 200 and 8 columns), which
# the solver leaves to the register-march kernel by default.
@pytest.mark.parametrize("shape,kind,order,always", [
    ((64, 20, 13), "aniso", "201", False),
    ((128, 20, 30), "aniso", "201", False),
    ((192, 9, 8), "iso", "012", False),
    ((248, 6, 7), "aniso", "120", False),
    ((36, 33, 21), "aniso", "201", True),
    ((40, 23, 17), "iso", "012", True),
    ((200, 12, 10), "aniso", "120", True),
    ((8, 9, 7), "iso", "210", True),
])
def test_cg_operator_matches_oracle_matrix(shape, kind, order, always, monkeypatch):
    if always:
        monkeypatch.setenv("PLGPU_TMA_ALWAYS", "1")
    if kind == "iso":
        s = S.layered_c0(seed=23, n=shape)
        s.convection = [("top", 50.0, 300.0)]
    else:
        s = S.layered_c1(seed=23, n=shape)
        s.heatflux = [("left", -2e4)]
        s.convection = s.convection + [("front", 20.0, 310.0)]
    sv = TH.solver_for_structure(s, ordering=order, algorithm="gpu-mixed")
    sv.compute(1)
    T = sv._full_temperature()
    p = O.from_structure(s, order=order)
    A, F, node_id, n = O.assemble(p, T)
    is_d, vf, vl = O.dirichlet_values(p, node_id, n)
    A2, _ = O.apply_dirichlet(A, F, is_d, vf, vl)
    rng = np.random.default_rng(9)
    x = rng.standard_normal(n)
    x[is_d] = 0.0  # the CG direction vanishes on Dirichlet nodes
    ref = A2 @ x
    y, xax, staged = sv._fem.cg_operator(x)
    assert staged, "the TMA-staged kernel should run on this mesh"
    free = ~is_d
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(y[free] - ref[free])) <= 2e-5 * scale
    ref_xax = float(x @ ref)
    assert abs(xax - ref_xax) <= 1e-5 * abs(ref_xax)


@pytest.mark.parametrize("n0", [35, 200])  # a row stride that is no multiple of 16 bytes; 78 % of the columns
def test_cg_operator_falls_back_on_unaligned_or_underfilled_meshes(n0):
    s = S.layered_c1(seed=24, n=(n0, 17, 12))
    sv = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    sv.compute(1)
    T = sv._full_temperature()
    p = O.from_structure(s, order="201")
    A, F, node_id, n = O.assemble(p, T)
    is_d, vf, vl = O.dirichlet_values(p, node_id, n)
    A2, _ = O.apply_dirichlet(A, F, is_d, vf, vl)
    x = np.random.default_rng(10).standard_normal(n)
    x[is_d] = 0.0
    ref = A2 @ x
    y, xax, staged = sv._fem.cg_operator(x)
    assert not staged
    free = ~is_d
    assert np.max(np.abs(y[free] - ref[free])) <= 2e-5 * np.max(np.abs(ref))
