"""Dynamic3D (theta-method time stepping, lumped or consistent heat capacity) on the GPU
against the CPU oracle (oracle/dynamic3d.py, a restatement of
solvers/thermal/dynamic/femT3d.cpp): temperatures within 1e-6 K after the same number of
steps, the same elapsed time, for Crank-Nicolson, implicit Euler, theta = 0.75, periodic
k(T) rebuilds and a second compute() that continues from the first.  Dirichlet nodes hold their values (the scheme the
reference's setMatrix prepares; its step loop lets them drift, see oracle/dynamic3d.py)."""
import numpy as np
import pytest

from oracle import dynamic3d as D
from oracle import fem3d as O
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu

TOL_T = 1e-6  # K


def _case(seed=5, n=(12, 11, 16)):
    s = S.layered_c0(seed=seed, n=n)
    rng = np.random.default_rng(seed + 77)
    cp = rng.uniform(300.0, 900.0, s.k300.size)
    dens = rng.uniform(2000.0, 7000.0, s.k300.size)
    return s, cp, dens


def _solver(s, cp, dens, order, **kw):
    sv = TH.Dynamic3D("dyn")
    g = TH.StructureGeometry.from_structure(s)
    g.materials.cp, g.materials.dens = cp, dens
    sv.geometry = g
    sv.mesh = TH.RectangularMesh3D(*s.axes, ordering=order)
    sv.inHeat = s.heat
    sv.algorithm = kw.pop("algorithm", "gpu-mixed")
    for side, v in s.temperature:
        sv.temperature_boundary.append(TH.RectangularMesh3D.side(side), v)
    for k, v in kw.items():
        setattr(sv, k, v)
    return sv


@pytest.mark.parametrize("theta,rebuild,algorithm,lumping", [
    (0.5, 0, "gpu-mixed", True), (1.0, 0, "gpu-pcg", True), (0.5, 3, "gpu-mixed", True),
    (0.5, 0, "gpu-mixed", False), (1.0, 2, "gpu-pcg", False), (0.75, 0, "gpu-mixed", False)])
def test_time_steps_match_oracle(theta, rebuild, algorithm, lumping):
    s, cp, dens = _case()
    order = "201"
    sv = _solver(s, cp, dens, order, timestep=0.2, methodparam=theta, rebuildfreq=rebuild, algorithm=algorithm,
                 lumping=lumping)
    sv.compute(2.0)
    p = O.from_structure(s, order=order, empty_elements="include")
    To, elaps, steps = D.compute(p, 2.0, cp, dens, timestep=0.2, theta=theta, lumping=lumping, rebuildfreq=rebuild)
    node_id, _ = O.masked_numbering(p)
    To_full = O.to_full(p, node_id, To)
    Tg = sv._full_temperature()
    print("steps", steps, sv.stats["loops"], "max |dT|", np.max(np.abs(Tg - To_full)), "max T", np.max(To),
          "bottom", float(np.max(np.abs(To_full[0] - 300.0))))
    assert sv.stats["loops"] == steps
    assert sv.time == pytest.approx(elaps, abs=1e-12)
    assert np.max(np.abs(Tg - To_full)) <= TOL_T
    assert np.max(To) > 300.5  # the source heated the structure


def test_second_compute_continues():
    s, cp, dens = _case(seed=6, n=(10, 12, 14))
    order = "012"
    sv = _solver(s, cp, dens, order, timestep=0.25)
    sv.compute(1.0)
    sv.compute(1.0)
    p = O.from_structure(s, order=order, empty_elements="include")
    T1, e1, _ = D.compute(p, 1.0, cp, dens, timestep=0.25)
    T2, e2, _ = D.compute(p, 1.0, cp, dens, T=T1, timestep=0.25)
    node_id, _ = O.masked_numbering(p)
    assert np.max(np.abs(sv._full_temperature() - O.to_full(p, node_id, T2))) <= TOL_T
    # elapsed time accumulates over calls (the reference keeps elapstime in the solver)
    assert sv.time == pytest.approx(e1 + e2, abs=1e-9)
