"""GPU solver against the FP64 oracle (band Cholesky, a restatement of therm3d.cpp).

Parity bar: max |dT| <= 1e-6 K against the oracle, the same number of outer
k(T) iterations, and the same toterr to 1e-6 K."""
import numpy as np
import pytest

from oracle import fem3d as O
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu

TOL_T = 1e-6  # K


def _gpu(s, order, algorithm, **kw):
    sv = TH.solver_for_structure(s, ordering=order, algorithm=algorithm, **kw)
    tot = sv.compute()
    return sv, sv._full_temperature(), tot


CASES = [
    ("c0", lambda: S.layered_c0(seed=3, n=(10, 12, 16)), "201"),
    ("c0-012", lambda: S.layered_c0(seed=4, n=(9, 9, 14)), "012"),
    ("c1", lambda: S.layered_c1(seed=5, n=(12, 10, 18)), "201"),
    ("c1-210", lambda: S.layered_c1(seed=6, n=(11, 13, 15)), "210"),
    # x-widths the TMA-staged operator and its CG take: one and two warps along x,
    # several row tiles and z-chunks
    ("c1-wide", lambda: S.layered_c1(seed=7, n=(64, 14, 20)), "201"),
    ("c0-wide", lambda: S.layered_c0(seed=9, n=(128, 10, 12)), "120"),
]


@pytest.mark.parametrize("algorithm", ["gpu-pcg", "gpu-mixed", "cholesky", "iterative"])
@pytest.mark.parametrize("name,make,order", CASES, ids=[c[0] for c in CASES])
def test_compute_matches_oracle(name, make, order, algorithm):
    s = make()
    To, tot_o, rec = O.compute(O.from_structure(s, order=order))
    sv, T, tot = _gpu(s, order, algorithm)
    assert sv.stats["loops"] == len(rec)
    assert np.max(np.abs(T - To)) <= TOL_T
    assert abs(tot - tot_o) <= TOL_T
    assert abs(sv.stats["max_t"] - rec[-1].maxT) <= TOL_T


def test_outer_iterations_one_by_one():
    """compute(1) repeatedly follows the oracle's loop body step by step (therm3d.cpp:311-333)."""
    s = S.layered_c1(seed=8, n=(10, 9, 15))
    order = "201"
    p = O.from_structure(s, order=order)
    sv = TH.solver_for_structure(s, ordering=order, algorithm="gpu-mixed")
    To = np.full(p.shape, 300.0)
    for loop in range(4):
        err = sv.compute(1)
        To_next, _ = O.outer_step(p, To)
        T = sv._full_temperature()
        assert np.max(np.abs(T - To_next)) <= TOL_T
        assert abs(err - np.max(np.abs(To_next - To))) <= TOL_T
        assert sv.stats["total_loops"] == loop + 1
        To = To_next


def test_heat_flux_conductivity_thickness_match_oracle():
    s = S.layered_c1(seed=9, n=(9, 11, 16))
    order = "201"
    p = O.from_structure(s, order=order)
    To, _, _ = O.compute(p)
    sv, T, _ = _gpu(s, order, "gpu-mixed")
    q_o = O.heat_fluxes(p, To)
    q = sv.heat_fluxes()
    scale = np.max(np.abs(q_o))
    assert np.max(np.abs(q - q_o)) <= 1e-6 * scale
    assert np.allclose(sv.thickness(), O.element_thickness(p), rtol=0, atol=1e-12)
    kxy, kz = O.element_k(p, To)
    k = sv.outThermalConductivity()
    # k = k300 (300/T)^p: |dk|/k <= p |dT| / T <= 1.5 * 1e-6 K / 300 K = 5e-9 at the temperature tolerance
    assert np.allclose(k[..., 0].ravel(), kxy, rtol=1e-8)
    assert np.allclose(k[..., 1].ravel(), kz, rtol=1e-8)


def _mesa_with_faces(seed, n):
    """A layered structure whose top layers are etched into a mesa (an EMPTY material
    around it: masked mesh), with heat flux, convection and radiation on several faces."""
    s = S.layered_c0(seed=seed, n=n, power=1e15)
    n_mat = s.k300.size
    s.k300 = np.append(s.k300, 0.026)
    s.p = np.append(s.p, 0.0)
    s.kz_ratio = np.append(s.kz_ratio, 1.0)
    s.hexp = np.append(s.hexp, 0.0)
    s.empty = np.append(s.empty, True)
    ne2 = s.mat.shape[0]
    xm = 0.5 * (s.axes[0][1:] + s.axes[0][:-1])
    ym = 0.5 * (s.axes[1][1:] + s.axes[1][:-1])
    outside = (xm[None, :] > 20.0) | (ym[:, None] > 20.0)
    mat = s.mat.copy()
    for k in range(ne2 - 4, ne2):
        mat[k][outside] = n_mat
    s.mat = mat
    s.heatflux = [("left", -2e3)]
    s.convection = [("top", 80.0, 295.0), ("right", 40.0, 300.0)]
    s.radiation = [("front", 0.7, 310.0), ("top", 0.5, 280.0)]
    return s


@pytest.mark.parametrize("algorithm,always", [("gpu-mixed", False), ("gpu-pcg", False), ("gpu-mixed", True)])
@pytest.mark.parametrize("order", ["201", "012"])
def test_masked_mesh_with_face_conditions_matches_oracle(order, algorithm, always, monkeypatch):
    """Full compute() with a masked mesh and heat-flux, convective and radiative faces in
    the reference's placement (face terms on element corners 0-3, radiation reading the
    temperatures of global nodes 0-7), against the oracle.  always: the TMA operator and
    its CG on this 12-column mesh too (surface rows on the top, right and front faces,
    masked-out nodes)."""
    if always:
        monkeypatch.setenv("PLGPU_TMA_ALWAYS", "1")
    s = _mesa_with_faces(seed=12, n=(12, 11, 16))
    p = O.from_structure(s, order=order)
    To, tot_o, rec = O.compute(p)
    sv, T, tot = _gpu(s, order, algorithm)
    node_id, n_act = O.masked_numbering(p)
    act = node_id >= 0
    assert n_act < act.size  # the etched corner drops nodes
    assert sv.stats["loops"] == len(rec)
    assert np.all(np.isnan(T[~act]))
    assert np.max(np.abs(T[act] - To[act])) <= TOL_T
    assert abs(tot - tot_o) <= TOL_T


@pytest.mark.parametrize("algorithm", ["gpu-mixed", "gpu-pcg"])
@pytest.mark.parametrize("seed", [2005, 2006])
def test_config2_structure_matches_oracle(seed, algorithm):
    """Structures of the learned preconditioner's configuration (random layers, a mesa etched
    through the upper ones: a masked mesh, an oxide aperture at 1e-2 of its host layer's
    conductivity, Gaussian heat blobs) at 24x24x32 nodes against the oracle's band
    Cholesky: the register-march operator's fused iteration (24 columns)."""
    s = S.learned_c2(seed=seed, n=(24, 24, 32))
    order = "201"
    p = O.from_structure(s, order=order)
    To, tot_o, rec = O.compute(p)
    sv, T, tot = _gpu(s, order, algorithm)
    act = O.masked_numbering(p)[0] >= 0
    assert not act.all()  # the etched region drops nodes
    assert sv.stats["loops"] == len(rec)
    assert np.max(np.abs(T[act] - To[act])) <= TOL_T
    assert abs(tot - tot_o) <= TOL_T
