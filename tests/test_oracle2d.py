"""CPU tests of the 2D FP64 oracle (oracle/fem2d.py, a restatement of
solvers/thermal/static/therm2d.cpp): analytic known answers that pin the
Cartesian and cylindrical assembly, the reference's own Static2D test (layer-run
thickness as the conductivity's second argument, solvers/thermal/static/tests/therm.py:47-53),
the masked numbering and the edge boundary terms."""
import numpy as np
import pytest

from oracle import fem2d as O2
from oracle import fem3d as O3
from plask_gb300 import structures as S


def _layered_slab(geometry="cartesian", order="01"):
    # four layers; heat in layer 2; bottom held at 300 K; laterally uniform
    y_layers = [0.0, 2.0, 2.5, 3.0, 5.0]
    cells = [3, 2, 2, 4]
    y = [0.0]
    mat_y = []
    for li, (a, b, c) in enumerate(zip(y_layers[:-1], y_layers[1:], cells)):
        for t in range(1, c + 1):
            y.append(a + (b - a) * t / c)
            mat_y.append(li)
    y = np.array(y)
    x = np.linspace(0.0, 6.0, 5) if geometry == "cartesian" else np.linspace(1.0, 7.0, 5)
    mat = np.broadcast_to(np.array(mat_y, np.int32)[:, None], (len(y) - 1, len(x) - 1)).copy()
    k300 = np.array([40.0, 3.0, 12.0, 70.0])
    q = np.zeros(mat.shape)
    q[mat == 2] = 5e15
    bottom = np.zeros((len(y), len(x)), bool)
    bottom[0] = True
    p = O2.Problem2D(axes=(x, y), mat=mat, materials=O3.Materials(k300, np.zeros(4)), heat=q, geometry=geometry,
                     temperature=[(bottom, 300.0)], order=order)
    return p, y, mat_y, k300, q


@pytest.mark.parametrize("order", ["01", "10"])
@pytest.mark.parametrize("geometry", ["cartesian", "cylindrical"])
def test_layered_slab_is_nodally_exact(order, geometry):
    """1D conduction through layers: the bilinear FEM gives the exact nodal temperatures
    (a laterally uniform field has no radial flux, so the cylindrical weight cancels)."""
    p, y, mat_y, k300, q = _layered_slab(geometry, order)
    T, _, _ = O2.compute(p, loops=1)
    qe = np.array([q[e, 0] for e in range(len(y) - 1)])
    dy = np.diff(y)
    # heat flowing down through each element's bottom face, per m^2
    Q = np.cumsum((qe * dy * 1e-6)[::-1])[::-1]
    exact = [300.0]
    for e in range(len(y) - 1):
        kk = k300[mat_y[e]]
        # T(y) within element e: quadratic; at the top node
        exact.append(exact[-1] + (Q[e] * dy[e] * 1e-6 - qe[e] * (dy[e] * 1e-6) ** 2 / 2) / kk)
    exact = np.array(exact)
    for col in range(T.shape[1]):
        np.testing.assert_allclose(T[:, col], exact, rtol=0, atol=1e-9)


def test_patch_linear_field_cartesian():
    """A linear field with Dirichlet values on the whole boundary is reproduced exactly."""
    x = np.array([0.0, 0.7, 1.5, 3.0, 3.2])
    y = np.array([0.0, 0.4, 1.0, 2.2])
    mat = np.zeros((3, 4), np.int32)
    mats = O3.Materials(np.array([5.0]), np.zeros(1), kz_ratio=np.array([0.6]))
    X, Y = np.meshgrid(x, y)
    field = 310.0 + 2.0 * X - 3.0 * Y
    bnd = np.zeros(X.shape, bool)
    bnd[0] = bnd[-1] = True
    bnd[:, 0] = bnd[:, -1] = True
    conds = [(np.where(bnd, True, False) & (X == xv) & (Y == yv), field[j, i])
             for j, yv in enumerate(y) for i, xv in enumerate(x) if bnd[j, i]]
    p = O2.Problem2D(axes=(x, y), mat=mat, materials=mats, heat=np.zeros(mat.shape), temperature=conds)
    # constant (anisotropic) conductivity: div(K grad T) = 0 for a linear T
    T, _, _ = O2.compute(p, loops=1)
    np.testing.assert_allclose(T, field, rtol=0, atol=1e-10)


def test_cylindrical_radial_conduction_converges_to_the_exact_profile():
    """Solid cylinder, uniform source, T(R) fixed: T(r) = T_R + q (R^2 - r^2) / (4 k) 1e-12."""
    R, k, qv = 20.0, 30.0, 1e16
    r = np.linspace(0.0, R, 161)
    y = np.array([0.0, 1.0])
    mat = np.zeros((1, len(r) - 1), np.int32)
    right = np.zeros((2, len(r)), bool)
    right[:, -1] = True
    p = O2.Problem2D(axes=(r, y), mat=mat, materials=O3.Materials(np.array([k]), np.zeros(1)),
                     heat=np.full(mat.shape, qv), geometry="cylindrical", temperature=[(right, 300.0)])
    T, _, _ = O2.compute(p, loops=1)
    exact = 300.0 + qv * (R ** 2 - r ** 2) / (4.0 * k) * 1e-12
    rise = exact[0] - 300.0
    assert np.max(np.abs(T[0] - exact)) <= 2e-4 * rise
    np.testing.assert_allclose(T[0], T[1], rtol=0, atol=1e-10)


def _strange_stack(order="01"):
    # GaAs-like 0.2 um, two 1 um "Strange" layers (thermk(T, h) = h), 0.2 um; 2 um wide
    y = np.array([0.0, 0.1, 0.2, 0.45, 0.7, 0.95, 1.2, 1.45, 1.7, 1.95, 2.2, 2.3, 2.4])
    x = np.linspace(0.0, 2.0, 5)
    lay = np.where((y[:-1] >= 0.2 - 1e-12) & (y[1:] <= 2.2 + 1e-12), 1, 0)
    mat = np.broadcast_to(lay[:, None], (len(y) - 1, len(x) - 1)).astype(np.int32).copy()
    mats = O3.Materials(np.array([44.0, 1.0]), np.array([1.25, 0.0]), hexp=np.array([0.0, 1.0]))
    bottom = np.zeros((len(y), len(x)), bool)
    bottom[0] = True
    return O2.Problem2D(axes=(x, y), mat=mat, materials=mats, heat=np.zeros(mat.shape),
                        temperature=[(bottom, 300.0)], order=order)


def test_reference_static2d_layer_thickness_conductivity():
    """solvers/thermal/static/tests/therm.py:47-53: two stacked 1 um layers of a material
    whose thermk(T, h) returns h make one 2 um run, so k = 2 at (1, 0.7) and (1, 1.7)."""
    p = _strange_stack()
    k = O2.conductivity(p, np.full(p.shape, 300.0))
    x, y = p.axes
    for px, py in ((1.0, 0.7), (1.0, 1.7)):
        i = np.searchsorted(x, px, side="left") - 1
        j = np.searchsorted(y, py, side="left") - 1
        assert k[j, i, 0] == pytest.approx(2.0, abs=1e-6)
        assert k[j, i, 1] == pytest.approx(2.0, abs=1e-6)


def test_masked_numbering_keeps_mesh_order():
    s = S.layered_2d(seed=4, n=(12, 16), etch=True)
    for order in ("01", "10"):
        p = O2.Problem2D(axes=s.axes, mat=s.mat, materials=O3.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty),
                         heat=s.heat, order=order)
        node_id, n = O2.masked_numbering(p)
        assert 0 < n < node_id.size
        ref = O2.reference_order(p.shape, order)
        act = node_id >= 0
        # masked ids increase with the full-mesh index
        ids = node_id[act]
        assert np.all(np.diff(ids[np.argsort(ref[act])]) == 1)


def test_convective_edge_terms_follow_the_reference_scaling():
    """Convection on the top edge, Cartesian: load 0.5e-6 len h Ta per node and stiffness
    (h1 + h2) len / 6 (diagonal), / 12 (off-diagonal) without the 1e-6 (bc_compat), or with it."""
    x = np.array([0.0, 2.0, 5.0])
    y = np.array([0.0, 1.0])
    mat = np.zeros((1, 2), np.int32)
    top = np.zeros((2, 3), bool)
    top[1] = True
    mats = O3.Materials(np.array([10.0]), np.zeros(1))
    for compat, scale in ((True, 1.0), (False, 1e-6)):
        p = O2.Problem2D(axes=(x, y), mat=mat, materials=mats, heat=np.zeros(mat.shape), convection=[(top, 7.0, 290.0)],
                         order="10", bc_compat=compat)
        A0, F0 = O2.assemble(O2.Problem2D(axes=(x, y), mat=mat, materials=mats, heat=np.zeros(mat.shape), order="10"),
                             np.full((2, 3), 300.0))
        A, F = O2.assemble(p, np.full((2, 3), 300.0))
        dA = (A - A0).toarray()
        n0 = 3
        t0, t1, t2 = n0, n0 + 1, n0 + 2  # top-row nodes in ORDER_10
        assert dA[t0, t0] == pytest.approx(scale * 14.0 * 2.0 / 6.0)
        assert dA[t1, t1] == pytest.approx(scale * 14.0 * (2.0 + 3.0) / 6.0)
        assert dA[t0, t1] == pytest.approx(scale * 14.0 * 2.0 / 12.0)
        assert dA[t1, t2] == pytest.approx(scale * 14.0 * 3.0 / 12.0)
        assert F[t1] - F0[t1] == pytest.approx(0.5e-6 * (2.0 + 3.0) * 7.0 * 290.0)


@pytest.mark.parametrize("geometry", ["cartesian", "cylindrical"])
@pytest.mark.parametrize("lumping", [True, False])
def test_dynamic2d_oracle_reaches_the_static_state(geometry, lumping):
    """Implicit Euler with a timestep far beyond the diffusion time, rebuilding k(T) every
    step, lands on the static 2D oracle's answer (solvers/thermal/dynamic/femT2d.cpp)."""
    from oracle import dynamic2d as D2

    s = S.layered_2d(seed=7, n=(14, 18))
    mats = O3.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty)
    bottom = np.zeros((len(s.axes[1]), len(s.axes[0])), bool)
    bottom[0] = True
    p = O2.Problem2D(axes=s.axes, mat=s.mat, materials=mats, heat=s.heat, geometry=geometry,
                     temperature=[(bottom, 300.0)], order="01")
    Ts, _, _ = O2.compute(p)
    cp = np.full(s.k300.size, 500.0)
    dens = np.full(s.k300.size, 5000.0)
    Td, elaps, steps = D2.compute(p, 10e9, cp, dens, timestep=1e9, theta=1.0, lumping=lumping, rebuildfreq=1)
    node_id, _ = O2.masked_numbering(p)
    assert steps == 11
    assert np.max(np.abs(O2.to_full(p, node_id, Td) - Ts)) < 0.1


def test_dynamic2d_consistent_capacity_rows_sum_to_lumped():
    from oracle import dynamic2d as D2

    s = S.layered_2d(seed=8, n=(9, 11))
    mats = O3.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty)
    for geometry in ("cartesian", "cylindrical"):
        p = O2.Problem2D(axes=s.axes, mat=s.mat, materials=mats, heat=s.heat, geometry=geometry)
        num = O2.masked_numbering(p)
        cp = np.linspace(300.0, 900.0, s.k300.size)
        dens = np.linspace(2000.0, 6000.0, s.k300.size)
        Cl = D2._mass(p, cp, dens, 0.1, True, num)
        Cc = D2._mass(p, cp, dens, 0.1, False, num)
        np.testing.assert_allclose(np.asarray(Cc.sum(axis=1)).ravel(), Cl.diagonal(), rtol=1e-13)
