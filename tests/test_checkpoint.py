"""Checkpoint / resume of the temperature field (plask_gb300.thermal.save_state and
load_state, the solvers' save() / load()): the reference keeps the temperatures between
compute() calls until invalidate() (solvers/thermal/static/therm3d.cpp:118-122); a saved
field restores that warm start in another solver object.  CPU: the mesh checks; GPU: the
round trip and the warm restart in 3D and 2D."""
import numpy as np
import pytest

from plask_gb300 import structures as S
from plask_gb300 import thermal as TH
from plask_gb300 import thermal2d as T2


def _fake_checkpoint(path, axes, ordering, n):
    data = {"temperature": np.full(n, 300.0), "ordering": np.array(ordering), "solver": np.array("Static3D")}
    for d, a in enumerate(axes):
        data[f"axis{d}"] = np.asarray(a, np.float64)
    np.savez(path, **data)


def test_load_rejects_another_mesh(tmp_path):
    s = S.layered_c0(seed=3, n=(8, 9, 10))
    sv = TH.solver_for_structure(s, ordering="012")
    f = tmp_path / "other.npz"
    axes = [a.copy() for a in s.axes]
    axes[2][-1] += 1.0
    _fake_checkpoint(f, axes, "012", 8 * 9 * 10)
    with pytest.raises(TH.BadInput, match="another mesh"):
        sv.load(f)
    g = tmp_path / "order.npz"
    _fake_checkpoint(g, s.axes, "210", 8 * 9 * 10)
    with pytest.raises(TH.BadInput, match="iteration order"):
        sv.load(g)
    h = tmp_path / "2d.npz"
    _fake_checkpoint(h, s.axes[:2], "012", 8 * 9)
    with pytest.raises(TH.BadInput, match="another mesh"):
        sv.load(h)


@pytest.mark.gpu
def test_round_trip_and_warm_restart_3d(tmp_path):
    s = S.layered_c0(seed=4, n=(12, 12, 16))
    a = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    a.compute()
    f = tmp_path / "t3d.npz"
    a.save(f)
    b = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    b.load(f)
    np.testing.assert_array_equal(b.temperatures(), a.temperatures())
    err = b.compute(1)  # starts from the converged field
    assert err <= b.maxerr
    assert b.stats["loops"] == 1
    assert np.max(np.abs(b._full_temperature() - a._full_temperature())) <= b.maxerr


@pytest.mark.gpu
def test_round_trip_masked_2d(tmp_path):
    s = S.layered_2d(seed=9, n=(20, 26), etch=True)
    a = T2.solver_for_structure2d(s, cls=T2.StaticCyl, ordering="10")
    a.compute()
    f = tmp_path / "t2d.npz"
    a.save(f)
    b = T2.solver_for_structure2d(s, cls=T2.StaticCyl, ordering="10")
    b.load(f)
    np.testing.assert_array_equal(b.temperatures(), a.temperatures())
    assert b.compute(1) <= b.maxerr
