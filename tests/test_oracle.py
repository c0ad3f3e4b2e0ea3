"""CPU tests of the FP64 oracle: analytic known answers that pin the assembly,
and the reference behaviours it restates (ordering, masking, boundary-face
placement, Dirichlet elimination order)."""
import numpy as np
import pytest

from oracle import fem3d as O


def _axes(n0, n1, z):
    return (np.linspace(0.0, 10.0, n0), np.linspace(0.0, 8.0, n1), np.asarray(z, float))


def _slab_problem(order="012"):
    # four layers of different conductivity; heat in layer 2; bottom held at 300 K
    z_layers = [0.0, 2.0, 2.5, 3.0, 5.0]
    cells = [3, 2, 2, 4]
    z = [0.0]
    mat_z = []
    for li, (a, b, c) in enumerate(zip(z_layers[:-1], z_layers[1:], cells)):
        for t in range(1, c + 1):
            z.append(a + (b - a) * t / c)
            mat_z.append(li)
    z = np.array(z)
    axes = _axes(3, 4, z)
    ne2 = len(z) - 1
    mat = np.broadcast_to(np.array(mat_z, np.int32)[:, None, None], (ne2, 3, 2)).copy()
    k300 = np.array([40.0, 3.0, 12.0, 70.0])
    mats = O.Materials(k300, np.zeros(4))
    q = np.zeros(mat.shape)
    q[mat == 2] = 5e15
    shape = (len(z), 4, 3)
    bottom = np.zeros(shape, bool)
    bottom[0] = True
    return O.Problem(axes=axes, mat=mat, materials=mats, heat=q, temperature=[(bottom, 300.0)], order=order), z, mat_z, k300, q


@pytest.mark.parametrize("order", ["012", "201", "120"])
def test_layered_slab_is_nodally_exact(order):
    """1D conduction through layers: trilinear FEM reproduces the exact nodal temperatures."""
    prob, z, mat_z, k300, q = _slab_problem(order)
    T, _, rec = O.compute(prob, loops=1)
    # exact: T(z) = 300 + int_0^z Phi(s)/k(s) ds, Phi(s) = heat flowing down through height s [W/m^2]
    qz = np.array([q[e, 0, 0] for e in range(len(mat_z))])
    dz = np.diff(z) * 1e-6
    phi_top = np.concatenate([np.cumsum((qz * dz)[::-1])[::-1][1:], [0.0]])  # flux through the top of each cell
    phi_bot = phi_top + qz * dz
    kz = k300[np.array(mat_z)]
    dT = dz * (phi_bot + phi_top) / (2 * kz)
    exact = 300.0 + np.concatenate([[0.0], np.cumsum(dT)])
    assert np.max(np.abs(T[:, 0, 0] - exact)) < 1e-9 * np.max(exact)
    assert np.max(np.abs(T - T[:, :1, :1])) < 1e-9  # laterally uniform


def test_patch_test_linear_field_reproduced():
    """A linear temperature field is an exact FEM solution for constant k and no source."""
    axes = (np.array([0.0, 0.7, 1.9, 3.0]), np.array([0.0, 1.1, 2.0, 2.4, 4.0]), np.array([0.0, 0.2, 1.5, 1.7, 3.0]))
    shape = tuple(len(a) for a in axes[::-1])
    Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    Tlin = 310.0 + 2.0 * X - 3.0 * Y + 5.0 * Z
    surface = np.zeros(shape, bool)
    surface[0] = surface[-1] = True
    surface[:, 0] = surface[:, -1] = True
    surface[:, :, 0] = surface[:, :, -1] = True
    bcs = []
    for idx in zip(*np.nonzero(surface)):
        m = np.zeros(shape, bool)
        m[idx] = True
        bcs.append((m, float(Tlin[idx])))
    mat = np.zeros(tuple(s - 1 for s in shape), np.int32)
    prob = O.Problem(axes=axes, mat=mat, materials=O.Materials([17.0], [0.0], [0.6]),
                     heat=np.zeros(mat.shape), temperature=bcs, order="201")
    T, _, _ = O.compute(prob, loops=1)
    assert np.max(np.abs(T - Tlin)) < 1e-9


def test_band_cholesky_matches_sparse_direct():
    from plask_gb300 import structures as S

    s = S.layered_c1(seed=7, n=(9, 8, 14))
    p = O.from_structure(s)
    Tc, _, rc = O.compute(p, method="cholesky")
    Td, _, rd = O.compute(p, method="direct")
    assert len(rc) == len(rd)
    assert np.max(np.abs(Tc - Td)) < 1e-8


def test_thickness_is_layer_run_height():
    """thermk(T, h) = h reports the height of the run of equal material (therm.py:47-53 analogue)."""
    z = np.array([0.0, 1.0, 2.0, 2.5, 3.0, 4.5, 6.0])
    mat_z = np.array([0, 0, 1, 1, 0, 2], np.int32)  # runs: [0,2) h=2, [2,4) h=1, [4,5) h=1.5, [5,6) h=1.5
    mat = np.broadcast_to(mat_z[:, None, None], (6, 2, 2)).copy()
    mat[4:, 1, 1] = 1  # a different column: run of material 1 from 2 to 6 minus ... -> [2,4) and [4,6) merge
    axes = _axes(3, 3, z)
    prob = O.Problem(axes=axes, mat=mat, materials=O.Materials([1.0, 1.0, 1.0], [0.0] * 3, hexp=[1.0] * 3),
                     heat=np.zeros(mat.shape))
    th = O.element_thickness(prob)
    assert np.allclose(th[:, 0, 0], [2.0, 2.0, 1.0, 1.0, 1.5, 1.5])
    assert np.allclose(th[:, 1, 1], [2.0, 2.0, 4.0, 4.0, 4.0, 4.0])
    kxy, kz = prob.materials.thermk(prob.mat.ravel(), np.full(mat.size, 300.0), th.ravel())
    assert np.allclose(kxy, th.ravel())


def test_reference_order_and_optimal_order():
    shape = (5, 4, 3)  # n2, n1, n0
    ref = O.reference_order(shape, "012")
    # axis 2 fastest: consecutive k at fixed (i, j)
    assert ref[1, 0, 0] - ref[0, 0, 0] == 1
    assert ref[0, 1, 0] - ref[0, 0, 0] == 5
    assert ref[0, 0, 1] - ref[0, 0, 0] == 20
    assert sorted(ref.ravel()) == list(range(60))
    assert O.optimal_order(40, 40, 60) == "201"
    assert O.optimal_order(128, 128, 200) == "201"
    assert O.optimal_order(60, 40, 40) == "012"


def test_masked_numbering_drops_empty_elements():
    z = np.linspace(0, 3, 4)
    axes = _axes(3, 3, z)
    mat = np.zeros((3, 2, 2), np.int32)
    mat[2] = 1  # top layer empty
    mat[1, 1, 1] = 1
    mats = O.Materials([10.0, 1.0], [0.0, 0.0], empty=[False, True])
    prob = O.Problem(axes=axes, mat=mat, materials=mats, heat=np.zeros(mat.shape), order="012")
    node_id, n_act = O.masked_numbering(prob)
    # the top plane is touched only by empty elements, and so is corner node (2, 2, 2)
    assert n_act == 26
    assert np.all(node_id[3] == -1) and node_id[2, 2, 2] == -1
    ids = node_id[node_id >= 0]
    assert sorted(ids) == list(range(n_act))
    ref = O.reference_order(prob.shape, "012")
    act = node_id >= 0
    assert np.all(np.argsort(ref[act]) == np.argsort(node_id[act]))
    prob_inc = O.Problem(axes=axes, mat=mat, materials=mats, heat=np.zeros(mat.shape), empty_elements="include")
    assert O.masked_numbering(prob_inc)[1] == 36


def _top_conv_problem(compat_axes=None):
    axes = _axes(3, 3, np.array([0.0, 1.0, 2.0]))
    shape = (3, 3, 3)
    mat = np.zeros((2, 2, 2), np.int32)
    top = np.zeros(shape, bool)
    top[-1] = True
    prob = O.Problem(axes=axes, mat=mat, materials=O.Materials([10.0], [0.0]), heat=np.zeros(mat.shape),
                     convection=[(top, 25.0, 320.0)], order="210")
    return prob


def test_face_terms_land_on_element_corners_0_to_3():
    """therm3d.cpp:150-165: a face's terms are added at the element's corners 0..3 (its z-lo face)."""
    prob = _top_conv_problem()
    T = np.full(prob.shape, 300.0)
    A, F, node_id, n = O.assemble(prob, T)
    base_noconv = O.Problem(axes=prob.axes, mat=prob.mat, materials=prob.materials, heat=prob.heat, order="210")
    A0, F0, _, _ = O.assemble(base_noconv, T)
    dFv = np.zeros(prob.shape)
    dFv.ravel()[:] = (F - F0)[node_id.ravel()]
    # nothing on the top plane, everything on the plane below it
    assert np.all(dFv[2] == 0.0)
    assert np.all(dFv[1] > 0.0)
    assert np.all(dFv[0] == 0.0)
    # total convective load = 0.25e-12 * area * h * Tamb summed per face corner
    area = 10.0 * 8.0
    assert np.isclose(dFv.sum(), 1e-12 * area * 25.0 * 320.0)
    dA = (A - A0).tocoo()
    rows = node_id.ravel()
    inv = np.empty(n, np.int64)
    inv[rows] = np.arange(rows.size)
    k_of = inv[dA.row] // 9
    assert set(np.unique(k_of[np.abs(dA.data) > 0])) == {1}


def test_radiation_reads_global_nodes_0_to_7():
    axes = _axes(3, 3, np.array([0.0, 1.0, 2.0]))
    shape = (3, 3, 3)
    top = np.zeros(shape, bool)
    top[-1] = True
    mat = np.zeros((2, 2, 2), np.int32)
    prob = O.Problem(axes=axes, mat=mat, materials=O.Materials([10.0], [0.0]), heat=np.zeros(mat.shape),
                     radiation=[(top, 0.8, 300.0)], order="210")
    T = np.full(shape, 300.0)
    _, F0, node_id, _ = O.assemble(prob, T)
    T2 = T.copy()
    T2[-1] = 500.0  # the radiating face itself is hot ...
    _, F2, _, _ = O.assemble(prob, T2)
    assert np.allclose(F0, 0.0) and np.allclose(F2, 0.0)  # ... but the term reads global nodes 0..7
    T3 = T.copy()
    ref = O.reference_order(shape, "210")
    T3.ravel()[np.flatnonzero(ref.ravel() < 8)] = 400.0
    _, F3, _, _ = O.assemble(prob, T3)
    assert np.all(F3 <= 0.0) and F3.min() < 0.0


def test_dirichlet_first_value_eliminates_last_value_stays():
    axes = _axes(3, 3, np.array([0.0, 1.0, 2.0]))
    shape = (3, 3, 3)
    bottom = np.zeros(shape, bool)
    bottom[0] = True
    corner = np.zeros(shape, bool)
    corner[0, 0, 0] = True
    mat = np.zeros((2, 2, 2), np.int32)
    prob = O.Problem(axes=axes, mat=mat, materials=O.Materials([10.0], [0.0]), heat=np.full(mat.shape, 1e15),
                     temperature=[(bottom, 300.0), (corner, 350.0)], order="012")
    node_id, n = O.masked_numbering(prob)
    is_d, vf, vl = O.dirichlet_values(prob, node_id, n)
    c = node_id[0, 0, 0]
    assert vf[c] == 300.0 and vl[c] == 350.0
    T, _, _ = O.compute(prob, loops=1)
    assert T[0, 0, 0] == 350.0
    assert np.all(T[0].ravel()[1:] == 300.0)


def test_heat_flux_of_slab_matches_power():
    prob, z, mat_z, k300, q = _slab_problem()
    T, _, _ = O.compute(prob, loops=1)
    flux = O.heat_fluxes(prob, T)
    # flux through the bottom cell equals the total heat per unit area, pointing down (-z)
    total = np.sum(q[:, 0, 0] * np.diff(z) * 1e-6)
    assert np.allclose(flux[0, :, :, 2], -total, rtol=1e-9)
    assert np.allclose(flux[..., :2], 0.0, atol=1e-6 * total)


@pytest.mark.parametrize("lumping", [True, False])
def test_dynamic_oracle_reaches_the_static_state(lumping):
    """Implicit Euler with a timestep far beyond the diffusion time, rebuilding k(T) every
    step, is a Picard iteration of the static problem: it must land on the static
    oracle's temperature (which itself stops at maxerr 0.05 K), with the lumped or the
    consistent heat capacity."""
    from oracle import dynamic3d as D
    from plask_gb300 import structures as S

    s = S.layered_c0(seed=21, n=(9, 8, 12))
    p = O.from_structure(s, order="012", empty_elements="include")
    Ts, _, _ = O.compute(p, loops=0)
    cp = np.full(s.k300.size, 500.0)
    dens = np.full(s.k300.size, 5000.0)
    Td, elaps, steps = D.compute(p, 10e9, cp, dens, timestep=1e9, theta=1.0, lumping=lumping, rebuildfreq=1,
                                 method="cholesky")
    node_id, _ = O.masked_numbering(p)
    assert steps == 11 and abs(elaps - 10e9) < 1e-3
    assert np.max(np.abs(O.to_full(p, node_id, Td) - Ts)) < 0.1


def test_consistent_capacity_rows_sum_to_the_lumped_capacity():
    """The consistent matrix c (8, 4, 2, 1)/27 per element (femT3d.cpp:203-226) has the
    lumped capacity as its row sums."""
    from oracle import dynamic3d as D
    from plask_gb300 import structures as S

    s = S.layered_c0(seed=22, n=(7, 6, 9))
    p = O.from_structure(s, order="012", empty_elements="include")
    numbering = O.masked_numbering(p)
    cp = np.linspace(300.0, 900.0, s.k300.size)
    dens = np.linspace(2000.0, 6000.0, s.k300.size)
    Cl = D._mass(p, cp, dens, 0.1, True, numbering)
    Cc = D._mass(p, cp, dens, 0.1, False, numbering)
    np.testing.assert_allclose(np.asarray(Cc.sum(axis=1)).ravel(), Cl.diagonal(), rtol=1e-13)
    assert abs(Cc - Cc.T).max() <= 1e-12 * abs(Cc).max()
