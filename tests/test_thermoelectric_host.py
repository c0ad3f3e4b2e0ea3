"""ThermoElectric3D's host-side helpers on the CPU, with stand-in solvers: the providers
it forwards, get_temperature / get_voltage / get_vertical_voltage and the field file of
save() (the fields of solvers/meta/shockley/thermoelectric.py:259-322 in an .npz file)."""
import numpy as np

from plask_gb300 import electrical as EL
from plask_gb300.mesh import RectangularMesh3D
from plask_gb300.thermal import Provider


class _Stand:
    def __init__(self, mesh, field):
        self.mesh = mesh
        self._field = field

    def _nodes(self, dst, interpolation="linear"):
        from plask_gb300.thermal import _points

        p = _points(dst)
        return self._field(p[:, 0], p[:, 1], p[:, 2])


def _te():
    tm = RectangularMesh3D(np.array([0.0, 1.0, 3.0]), np.array([0.0, 2.0]), np.array([0.0, 1.0, 2.0, 4.0]),
                           ordering="201")
    vm = RectangularMesh3D(np.array([0.0, 1.0, 3.0]), np.array([0.0, 2.0]), np.array([0.0, 1.0, 2.0, 4.0]),
                           ordering="012")
    te = EL.ThermoElectric3D()
    th = _Stand(tm, lambda x, y, z: 300.0 + x + 10 * y + 100 * z)
    th.outTemperature = Provider(th._nodes)
    el = _Stand(vm, lambda x, y, z: 2.0 - 0.1 * z + 0 * x)
    el.outVoltage = Provider(el._nodes)
    jz = np.arange(vm.elements_count, dtype=float)
    el.outCurrentDensity = Provider(lambda dst, interpolation="linear": np.stack(
        [np.zeros_like(jz), np.zeros_like(jz), jz], axis=-1).reshape(vm.element_shape + (3,)))
    te.thermal, te.electrical = th, el
    return te, tm, vm


def test_fields_and_forwarded_providers():
    te, tm, vm = _te()
    assert te.outTemperature is te.thermal.outTemperature and te.outVoltage is te.electrical.outVoltage
    T = te.get_temperature()
    assert T.shape == (len(tm),)
    v = te.get_vertical_voltage(at=(1.0, 2.0))
    np.testing.assert_allclose(v, 2.0 - 0.1 * vm.axis2)


def test_save_writes_the_fields_in_canonical_order(tmp_path):
    te, tm, vm = _te()
    f = te.save(tmp_path / "te.npz", group="Run")
    with np.load(f) as d:
        T = d["Run/Temperature"]
        assert T.shape == tm.shape
        z, y, x = np.meshgrid(tm.axis2, tm.axis1, tm.axis0, indexing="ij")
        np.testing.assert_allclose(T, 300.0 + x + 10 * y + 100 * z)
        np.testing.assert_allclose(d["Run/Potential"], 2.0 - 0.1 * np.meshgrid(vm.axis2, vm.axis1, vm.axis0,
                                                                               indexing="ij")[0])
        assert d["Run/CurrentDensity"].shape == vm.element_shape + (3,)
        np.testing.assert_allclose(d["Run/CurrentDensity/axis2"], 0.5 * (vm.axis2[1:] + vm.axis2[:-1]))
        assert str(d["Run/Temperature/ordering"]) == "201"
