"""Static2D / StaticCyl on the GPU (planar handles, include/plgpu_fem2d.h) against the
2D CPU oracle (oracle/fem2d.py, a restatement of solvers/thermal/static/therm2d.cpp):
temperatures within 1e-6 K after the full k(T) loop for both geometries, both
iteration orders, masked meshes, anisotropy, and heat-flux / convection / radiation
edge conditions in both placements; the operator against the assembled matrix; heat
fluxes; the reference's own Static2D conductivity test (tests/therm.py:47-53); Dynamic2D /
DynamicCyl time steps against oracle/dynamic2d.py (solvers/thermal/dynamic/femT2d.cpp)."""
import numpy as np
import pytest

from oracle import fem2d as O2
from oracle import fem3d as O3
from plask_gb300 import _native
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH
from plask_gb300 import thermal2d as T2

pytestmark = pytest.mark.gpu

TOL_T = 1e-6  # K


def _oracle_problem(s, sv, **kw):
    mats = O3.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty)
    shape = (len(s.axes[1]), len(s.axes[0]))

    def place(side):
        return T2.RectangularMesh2D.side(side).mask(sv.mesh)

    return O2.Problem2D(axes=s.axes, mat=s.mat, materials=mats, heat=s.heat, geometry=sv._geometry_kind,
                        temperature=[(place(a), v) for a, v in s.temperature],
                        heatflux=[(place(a), v) for a, v in s.heatflux],
                        convection=[(place(a), h, t) for a, h, t in s.convection],
                        radiation=[(place(a), e, t) for a, e, t in s.radiation],
                        order=sv.mesh.ordering, inittemp=s.inittemp, maxerr=s.maxerr,
                        empty_elements="exclude" if sv.empty_elements in ("default", "exclude") else "include",
                        bc_compat=sv.bc_compat, **kw)


CASES = [
    # (geometry class, seed, n, order, etch, aniso, algorithm)
    (T2.Static2D, 11, (40, 60), "01", False, False, "gpu-mixed"),
    (T2.Static2D, 12, (33, 47), "10", True, True, "gpu-mixed"),
    (T2.Static2D, 13, (30, 41), "01", False, True, "gpu-pcg"),
    (T2.StaticCyl, 21, (40, 60), "10", False, False, "gpu-mixed"),
    (T2.StaticCyl, 22, (35, 52), "01", True, True, "gpu-mixed"),
    (T2.StaticCyl, 23, (28, 44), "10", False, False, "gpu-pcg"),
]


@pytest.mark.parametrize("cls,seed,n,order,etch,aniso,algorithm", CASES)
def test_static_solve_matches_oracle(cls, seed, n, order, etch, aniso, algorithm):
    s = S.layered_2d(seed=seed, n=n, etch=etch, anisotropic=aniso)
    sv = T2.solver_for_structure2d(s, cls=cls, ordering=order, algorithm=algorithm)
    tot = sv.compute()
    p = _oracle_problem(s, sv)
    To, toterr, rec = O2.compute(p)
    Tg = sv._full_temperature()
    act = O2.masked_numbering(p)[0] >= 0
    d = np.max(np.abs(Tg[act] - To[act]))
    print(cls.__name__, seed, "loops", sv.stats["loops"], len(rec), "max|dT|", d, "maxT", np.nanmax(To))
    assert np.all(np.isnan(Tg[~act]))
    assert d <= TOL_T
    assert sv.stats["loops"] == len(rec)
    assert tot == pytest.approx(toterr, abs=1e-5)
    assert np.nanmax(To) > 301.0


@pytest.mark.parametrize("cls", [T2.Static2D, T2.StaticCyl])
@pytest.mark.parametrize("bc_compat", [True, False])
def test_edge_conditions_match_oracle(cls, bc_compat):
    """Heat flux on the right edge, convection and radiation on the top edge (first match
    per node), a Dirichlet bottom: both placements of the convective stiffness.  The
    reference's placement (bc_compat) has a stiffness 1e6 times its load term, which pulls
    the edge toward 1e-6 T_amb; a small coefficient keeps that edge near room temperature."""
    s = S.layered_2d(seed=31, n=(30, 40))
    s.heatflux = [("right", -2e5)]
    s.convection = [("top", 1e-3 if bc_compat else 1e4, 290.0)]
    s.radiation = [("top", 0.8, 280.0)]
    sv = T2.solver_for_structure2d(s, cls=cls, ordering="01", bc_compat=bc_compat)
    sv.compute(3)
    p = _oracle_problem(s, sv)
    To, _, _ = O2.compute(p, loops=3)
    d = np.max(np.abs(sv._full_temperature() - To))
    assert np.isfinite(d)
    print(cls.__name__, bc_compat, "max|dT|", d, "T range", To.min(), To.max())
    assert d <= TOL_T


@pytest.mark.parametrize("cls", [T2.Static2D, T2.StaticCyl])
def test_operator_matches_assembled_matrix(cls):
    s = S.layered_2d(seed=41, n=(21, 27), etch=True, anisotropic=True)
    s.convection = [("top", 3e3, 300.0)]
    sv = T2.solver_for_structure2d(s, cls=cls, ordering="10", empty_elements="include")
    sv.initialize()
    fem = sv._fem
    rng = np.random.default_rng(5)
    x = 300.0 + rng.standard_normal(len(sv.mesh))
    y64 = fem.mult(x, 64)
    y32 = fem.mult(x, 32)
    p = _oracle_problem(s, sv)
    node_id, n = O2.masked_numbering(p)
    assert n == len(sv.mesh)
    A, Fv = O2.assemble(p, np.full(p.shape, 300.0), numbering=(node_id, n))
    is_d, vf, vl = O2.dirichlet_values(p, node_id, n)
    A2, _ = O3.apply_dirichlet(A, Fv, is_d, vf, vl)
    # mesh-order x -> masked (== mesh order here) numbering
    ref = A2 @ x
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(y64 - ref)) <= 1e-12 * scale
    assert np.max(np.abs(y32 - ref)) <= 2e-5 * scale


@pytest.mark.parametrize("cls", [T2.Static2D, T2.StaticCyl])
def test_heat_fluxes_and_conductivity_match_oracle(cls):
    s = S.layered_2d(seed=51, n=(25, 35), anisotropic=True)
    sv = T2.solver_for_structure2d(s, cls=cls, ordering="01")
    sv.compute()
    p = _oracle_problem(s, sv)
    T = sv._full_temperature()
    q = sv.heat_fluxes()
    qo = O2.heat_fluxes(p, T)
    assert np.max(np.abs(q - qo)) <= 1e-9 * np.max(np.abs(qo))
    k = sv.outThermalConductivity(None)
    ko = O2.conductivity(p, T)
    np.testing.assert_allclose(k, ko, rtol=1e-12)
    th = sv.thickness()
    np.testing.assert_allclose(th, O2.element_thickness(p), rtol=0, atol=1e-12)


def test_reference_static2d_layer_thickness_conductivity():
    """solvers/thermal/static/tests/therm.py:47-53 through the GPU solver's provider."""
    y = np.array([0.0, 0.1, 0.2, 0.45, 0.7, 0.95, 1.2, 1.45, 1.7, 1.95, 2.2, 2.3, 2.4])
    x = np.linspace(0.0, 2.0, 5)
    lay = np.where((y[:-1] >= 0.2 - 1e-12) & (y[1:] <= 2.2 + 1e-12), 1, 0)
    mat = np.broadcast_to(lay[:, None], (len(y) - 1, len(x) - 1)).astype(np.int32).copy()
    sv = T2.Static2D("therm2d")
    sv.geometry = T2.StructureGeometry2D(TH.MaterialTable(np.array([44.0, 1.0]), np.array([1.25, 0.0]),
                                                          hexp=np.array([0.0, 1.0])), mat=mat)
    sv.mesh = T2.RectangularMesh2D(x, y)
    conds = sv.outThermalConductivity(np.array([[1.0, 0.7], [1.0, 1.7]]))
    assert conds[0][0] == pytest.approx(2.0, abs=1e-6)
    assert conds[1][0] == pytest.approx(2.0, abs=1e-6)


DYN_CASES = [
    # (class, seed, n, order, etch, aniso, theta, rebuildfreq, algorithm, lumping)
    (T2.Dynamic2D, 71, (24, 30), "01", False, True, 0.5, 0, "gpu-mixed", True),
    (T2.Dynamic2D, 72, (21, 33), "10", True, False, 1.0, 2, "gpu-pcg", False),
    (T2.DynamicCyl, 73, (24, 30), "10", False, False, 0.5, 3, "gpu-mixed", True),
    (T2.DynamicCyl, 74, (22, 28), "01", True, True, 0.75, 0, "gpu-mixed", False),
]


@pytest.mark.parametrize("cls,seed,n,order,etch,aniso,theta,rebuild,algorithm,lumping", DYN_CASES)
def test_time_steps_match_oracle(cls, seed, n, order, etch, aniso, theta, rebuild, algorithm, lumping):
    """Dynamic2D / DynamicCyl against oracle/dynamic2d.py (femT2d.cpp): the same steps and
    elapsed time, temperatures within 1e-6 K, lumped and consistent capacity, masked meshes."""
    from oracle import dynamic2d as D2

    s = S.layered_2d(seed=seed, n=n, etch=etch, anisotropic=aniso)
    s.heatflux, s.convection, s.radiation = [], [], []
    rng = np.random.default_rng(seed)
    cp = rng.uniform(300.0, 900.0, s.k300.size)
    dens = rng.uniform(2000.0, 7000.0, s.k300.size)
    sv = T2.solver_for_structure2d(s, cls=cls, ordering=order, algorithm=algorithm, timestep=0.2,
                                   methodparam=theta, rebuildfreq=rebuild, lumping=lumping)
    sv.geometry.materials.cp, sv.geometry.materials.dens = cp, dens
    sv.compute(2.0)
    p = _oracle_problem(s, sv)
    To, elaps, steps = D2.compute(p, 2.0, cp, dens, timestep=0.2, theta=theta, lumping=lumping, rebuildfreq=rebuild)
    node_id, _ = O2.masked_numbering(p)
    To_full = O2.to_full(p, node_id, To, fill=np.nan)
    Tg = sv._full_temperature()
    act = node_id >= 0
    d = np.max(np.abs(Tg[act] - To_full[act]))
    print(cls.__name__, seed, "steps", steps, sv.stats["loops"], "max|dT|", d, "maxT", np.max(To))
    assert np.all(np.isnan(Tg[~act]))
    assert sv.stats["loops"] == steps
    assert sv.time == pytest.approx(elaps, abs=1e-12)
    assert d <= TOL_T
    assert np.max(To) > 300.2  # the source heated the structure


def test_time_stepping_takes_temperature_conditions_only():
    s = S.layered_2d(seed=3, n=(10, 12))
    sv = T2.solver_for_structure2d(s, cls=T2.Dynamic2D)
    sv.geometry.materials.cp = np.ones(s.k300.size)
    sv.geometry.materials.dens = np.ones(s.k300.size)
    sv.initialize()
    sv._fem.add_bc(_native.BC_HEATFLUX, np.array([0, 1]), 1e5)
    with pytest.raises(_native.NativeError):
        sv._fem.set_dynamic(np.ones(s.k300.size), np.ones(s.k300.size))
        sv._fem.compute_dynamic(1.0)


@pytest.mark.parametrize("cls", [T2.Static2D, T2.StaticCyl])
def test_nearest_interpolation_of_providers(cls):
    s = S.layered_2d(seed=61, n=(20, 26))
    sv = T2.solver_for_structure2d(s, cls=cls, ordering="10")
    sv.compute()
    T = sv._full_temperature()
    x0, x1 = sv.mesh.axes
    # at the nodes, nearest and linear give the nodal temperature
    pts = np.array([[x0[3], x1[5]], [x0[-1], x1[0]]])
    np.testing.assert_allclose(sv.outTemperature(pts, "nearest"), [T[5, 3], T[0, -1]], rtol=0, atol=0)
    # just right of a node the nearest node is that node
    p = np.array([[x0[3] + 0.25 * (x0[4] - x0[3]), x1[5]]])
    assert sv.outTemperature(p, "nearest")[0] == T[5, 3]
    q = sv.heat_fluxes()
    mid = np.array([[0.5 * (x0[2] + x0[3]), 0.5 * (x1[7] + x1[8])]])
    np.testing.assert_allclose(sv.outHeatFlux(mid, "nearest")[0], q[7, 2])
