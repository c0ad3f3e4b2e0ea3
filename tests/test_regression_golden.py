"""Golden fixtures (tests/golden, written by tests/golden/make_golden.py): small seeded
problems with the answers of the reference path stored beside them.

CPU: the oracle replays every fixture to 1e-9 (its own answers, pinned against drift),
and its Static3D temperatures agree with the reference's own NSPCG solver (compiled from
the reference tree when the fixture was made) to 1e-8 K.  GPU: the CUDA path reproduces
every stored answer within the parity bar (1e-6 K, 1e-9 V) with the same loop count."""
import pathlib
import sys

import numpy as np
import pytest

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent / "golden"))

import golden_io as G  # noqa: E402
from oracle import dynamic2d as D2  # noqa: E402
from oracle import dynamic3d as D3  # noqa: E402
from oracle import electr3d as E  # noqa: E402
from oracle import fem2d as O2  # noqa: E402
from oracle import fem3d as O  # noqa: E402
from plask_gb300.mesh import RectangularMesh2D  # noqa: E402

TOL_T = 1e-6  # K
TOL_V = 1e-9  # V
FIXTURES = G.names()


def _element_mean(T):
    """Element-average temperatures (the 8-node mean) of a canonical node field."""
    return 0.125 * (T[:-1, :-1, :-1] + T[:-1, :-1, 1:] + T[:-1, 1:, :-1] + T[:-1, 1:, 1:]
                    + T[1:, :-1, :-1] + T[1:, :-1, 1:] + T[1:, 1:, :-1] + T[1:, 1:, 1:])


def _elec_structure(data, meta):
    """An electrical fixture's structure; a stored beta(T) = b0 (300/T)^bp becomes the callable
    the solvers evaluate at the element temperatures (electr_python.cpp:104-111)."""
    s = G.unpack_elec(data, meta)
    if meta.get("beta_T"):
        b0, bp = meta["beta_T"]
        s.beta = [lambda T, b0=b0, bp=bp: b0 * (300.0 / T) ** bp for _ in s.beta]
    return s


def _problem2d(s, meta):
    mats = O.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty)
    mesh = RectangularMesh2D(*s.axes, ordering=meta["order"])

    def place(side):
        return RectangularMesh2D.side(side).mask(mesh)

    return O2.Problem2D(axes=s.axes, mat=s.mat, materials=mats, heat=s.heat, geometry=meta["geometry"],
                        temperature=[(place(a), v) for a, v in s.temperature],
                        heatflux=[(place(a), v) for a, v in s.heatflux],
                        convection=[(place(a), h, t) for a, h, t in s.convection],
                        radiation=[(place(a), e, t) for a, e, t in s.radiation],
                        order=meta["order"], inittemp=s.inittemp, maxerr=s.maxerr,
                        empty_elements=meta["empty_elements"], bc_compat=meta["bc_compat"])


def _same_nan(a, b):
    return np.array_equal(np.isnan(a), np.isnan(b))


def _maxdiff(a, b):
    ok = ~np.isnan(b)
    return float(np.max(np.abs(a[ok] - b[ok])))


def test_fixtures_present():
    assert len(FIXTURES) >= 5


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_replays_fixture(name):
    data, meta = G.load(name)
    kind = meta["kind"]
    if kind == "static3d":
        s = G.unpack_thermal(data, meta)
        T, toterr, rec = O.compute(O.from_structure(s, order=meta["order"], empty_elements=meta["empty_elements"]))
        ref = data["T_cholesky"]
        assert _same_nan(T, ref) and _maxdiff(T, ref) <= 1e-9
        assert len(rec) == len(meta["records"]) and toterr == pytest.approx(meta["toterr"], abs=1e-9)
    elif kind == "static2d":
        s = G.unpack_thermal(data, meta)
        T, toterr, rec = O2.compute(_problem2d(s, meta))
        ref = data["T_cholesky"]
        assert _same_nan(T, ref) and _maxdiff(T, ref) <= 1e-9
        assert len(rec) == len(meta["records"]) and toterr == pytest.approx(meta["toterr"], abs=1e-9)
    elif kind == "dynamic3d":
        s = G.unpack_thermal(data, meta)
        p = O.from_structure(s, order=meta["order"], empty_elements=meta["empty_elements"])
        T, elaps, steps = D3.compute(p, meta["time"], data["cp"], data["dens"], timestep=meta["timestep"],
                                     theta=meta["theta"], lumping=meta["lumping"], rebuildfreq=meta["rebuildfreq"])
        node_id, _ = O.masked_numbering(p)
        assert _maxdiff(O.to_full(p, node_id, T), data["T_direct"]) <= 1e-9
        assert steps == meta["steps"] and elaps == pytest.approx(meta["elapsed"], abs=1e-12)
    elif kind == "dynamic2d":
        s = G.unpack_thermal(data, meta)
        p = _problem2d(s, meta)
        T, elaps, steps = D2.compute(p, meta["time"], data["cp"], data["dens"], timestep=meta["timestep"],
                                     theta=meta["theta"], lumping=meta["lumping"], rebuildfreq=meta["rebuildfreq"])
        node_id, _ = O2.masked_numbering(p)
        T = O2.to_full(p, node_id, T, fill=np.nan)
        assert _same_nan(T, data["T_direct"]) and _maxdiff(T, data["T_direct"]) <= 1e-9
        assert steps == meta["steps"] and elaps == pytest.approx(meta["elapsed"], abs=1e-12)
    elif kind == "thermoelectric3d":
        s = _elec_structure(data, meta)
        p = E.from_structure(s, order=meta["order"])
        tp = O.from_structure(s.thermal, order=meta["order"])
        state, T, n = {}, None, 0
        ve, tt = 2 * s.maxerr, 2 * tp.maxerr
        while tt > tp.maxerr or ve > s.maxerr:
            # the electrical problem reads the last thermal solve's element temperatures
            p.temperature = np.full(tuple(k - 1 for k in tp.shape), tp.inittemp) if T is None else _element_mean(T)
            V, conds, ve, _ = E.compute(p, loops=meta["tfreq"], state=state)
            tp.heat = E.heat(p, V, conds)
            T, tt, _ = O.compute(tp, loops=1, T=T)
            n += 1
        assert n == len(meta["rounds"])
        assert _maxdiff(T, data["T_cholesky"]) <= 1e-9 and _maxdiff(V, data["V_cholesky"]) <= 1e-12
    elif kind == "shockley3d":
        s = G.unpack_elec(data, meta)
        p = E.from_structure(s, order=meta["order"], convergence=meta["convergence"])
        V, conds, toterr, _ = E.compute(p, loops=meta["loops"])
        assert _maxdiff(V, data["V_cholesky"]) <= 1e-12
        assert toterr == pytest.approx(meta["toterr"], rel=1e-9)
    else:
        pytest.fail(f"unknown fixture kind {kind}")


def test_oracle_agrees_with_the_reference_nspcg():
    """The oracle's Static3D loop against the reference's own iterative solver (NSPCG,
    IC-CG, zeta 1e-12) on the same assembled systems, as stored in the fixture."""
    data, meta = G.load("static3d_layered_aniso_12x10x18")
    s = G.unpack_thermal(data, meta)
    T, _, rec = O.compute(O.from_structure(s, order=meta["order"]))
    assert _maxdiff(T, data["T_nspcg"]) <= 1e-8
    assert len(rec) == len(meta["nspcg"]["records"])
    assert all(0 < it < 5000 for it in meta["nspcg"]["iterations"])  # every NSPCG solve converged


# ----------------------------------------------------------------------------- GPU


def _gpu_static3d(data, meta, algorithm):
    from plask_gb300 import thermal as TH

    s = G.unpack_thermal(data, meta)
    sv = TH.solver_for_structure(s, ordering=meta["order"], algorithm=algorithm)
    tot = sv.compute()
    # nodes of the masked mesh (the oracle keeps the others at their initial value, the
    # solver reports NaN there)
    p = O.from_structure(s, order=meta["order"], empty_elements=meta["empty_elements"])
    act = O.masked_numbering(p)[0] >= 0
    return sv, sv._full_temperature(), tot, act


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", ["gpu-mixed", "gpu-pcg"])
@pytest.mark.parametrize("name", ["static3d_layered_aniso_12x10x18", "static3d_mesa_faces_12x11x16"])
def test_gpu_static3d_matches_fixture(name, algorithm):
    data, meta = G.load(name)
    sv, T, tot, act = _gpu_static3d(data, meta, algorithm)
    ref = data["T_cholesky"]
    assert np.all(np.isnan(T[~act]))
    assert np.max(np.abs(T[act] - ref[act])) <= TOL_T
    assert sv.stats["loops"] == len(meta["records"])
    assert abs(tot - meta["toterr"]) <= TOL_T
    if "T_nspcg" in data:
        assert np.max(np.abs(T[act] - data["T_nspcg"][act])) <= TOL_T


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["staticcyl_etched_aniso_35x52", "static2d_etched_aniso_33x47"])
def test_gpu_static2d_matches_fixture(name):
    from plask_gb300 import thermal2d as T2

    data, meta = G.load(name)
    s = G.unpack_thermal(data, meta)
    cls = T2.StaticCyl if meta["geometry"] == "cylindrical" else T2.Static2D
    sv = T2.solver_for_structure2d(s, cls=cls, ordering=meta["order"], bc_compat=meta["bc_compat"])
    tot = sv.compute()
    T = sv._full_temperature()
    ref = data["T_cholesky"]
    act = O2.masked_numbering(_problem2d(s, meta))[0] >= 0
    assert np.all(np.isnan(T[~act]))
    assert np.max(np.abs(T[act] - ref[act])) <= TOL_T
    assert sv.stats["loops"] == len(meta["records"])
    assert tot == pytest.approx(meta["toterr"], abs=1e-5)


@pytest.mark.gpu
def test_gpu_dynamic3d_matches_fixture():
    from plask_gb300 import thermal as TH

    data, meta = G.load("dynamic3d_consistent_12x11x16")
    s = G.unpack_thermal(data, meta)
    sv = TH.Dynamic3D("golden")
    g = TH.StructureGeometry.from_structure(s)
    g.materials.cp, g.materials.dens = data["cp"], data["dens"]
    sv.geometry = g
    sv.mesh = TH.RectangularMesh3D(*s.axes, ordering=meta["order"])
    sv.inHeat = s.heat
    sv.algorithm = "gpu-mixed"
    for side, v in s.temperature:
        sv.temperature_boundary.append(TH.RectangularMesh3D.side(side), v)
    sv.timestep, sv.methodparam, sv.lumping = meta["timestep"], meta["theta"], meta["lumping"]
    sv.compute(meta["time"])
    assert sv.stats["loops"] == meta["steps"]
    assert sv.time == pytest.approx(meta["elapsed"], abs=1e-12)
    assert _maxdiff(sv._full_temperature(), data["T_direct"]) <= TOL_T


@pytest.mark.gpu
def test_gpu_dynamiccyl_matches_fixture():
    from plask_gb300 import thermal2d as T2

    data, meta = G.load("dynamiccyl_lumped_24x30")
    s = G.unpack_thermal(data, meta)
    sv = T2.solver_for_structure2d(s, cls=T2.DynamicCyl, ordering=meta["order"], algorithm="gpu-mixed",
                                   timestep=meta["timestep"], methodparam=meta["theta"],
                                   rebuildfreq=meta["rebuildfreq"], lumping=meta["lumping"])
    sv.geometry.materials.cp, sv.geometry.materials.dens = data["cp"], data["dens"]
    sv.compute(meta["time"])
    T = sv._full_temperature()
    ref = data["T_direct"]
    assert _same_nan(T, ref)
    assert _maxdiff(T, ref) <= TOL_T
    assert sv.stats["loops"] == meta["steps"]
    assert sv.time == pytest.approx(meta["elapsed"], abs=1e-12)


@pytest.mark.gpu
def test_gpu_shockley3d_matches_fixture():
    from plask_gb300 import electrical as EL

    data, meta = G.load("shockley3d_junction_21x19x30")
    s = G.unpack_elec(data, meta)
    sv = EL.solver_for_structure(s, ordering=meta["order"], algorithm="gpu-mixed", convergence=meta["convergence"])
    sv.compute(meta["loops"])
    assert _maxdiff(sv._full_potential(), data["V_cholesky"]) <= TOL_V
    assert sv.err == pytest.approx(meta["toterr"], rel=1e-6)
    assert sv.get_total_current() == pytest.approx(meta["total_current"], rel=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["thermoelectric3d_19x19x28", "thermoelectric3d_betaT_19x19x28"])
def test_gpu_thermoelectric3d_matches_fixture(name):
    from plask_gb300 import electrical as EL
    from plask_gb300 import thermal as TH

    data, meta = G.load(name)
    s = _elec_structure(data, meta)
    te = EL.ThermoElectric3D()
    te.thermal = TH.solver_for_structure(s.thermal, ordering=meta["order"], algorithm="gpu-mixed")
    te.electrical = EL.solver_for_structure(s, ordering=meta["order"], algorithm="gpu-mixed")
    te.reconnect()
    verr, terr = te.compute()
    assert verr <= te.electrical.maxerr and terr <= te.thermal.maxerr
    assert len(te.history) == len(meta["rounds"])
    assert _maxdiff(te.thermal._full_temperature(), data["T_cholesky"]) <= TOL_T
    assert _maxdiff(te.electrical._full_potential(), data["V_cholesky"]) <= TOL_V
