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
