"""Provider helpers on the CPU: the nearest-node rule of PLaSK's rectilinear meshes
(find_nearest_binary, plask/utils/stl.hpp:59-80: the lower node on a tie, clamped to the
axis) and the element lookup (findUpIndex - 1, clamped)."""
import numpy as np
import pytest

from plask_gb300.thermal import BadInput, _check_interpolation, _element_axis, _nearest_axis, conductivity_elements


def test_nearest_node_rule():
    a = np.array([0.0, 1.0, 3.0, 4.0])
    x = np.array([-1.0, 0.0, 0.5, 0.6, 2.0, 2.1, 3.5, 5.0])
    assert list(_nearest_axis(a, x)) == [0, 0, 0, 1, 1, 2, 2, 3]


def test_element_lookup():
    a = np.array([0.0, 1.0, 3.0, 4.0])
    x = np.array([-1.0, 0.0, 0.5, 1.0, 3.9, 4.0, 5.0])
    assert list(_element_axis(a, x)) == [0, 0, 0, 1, 2, 2, 2]


def test_interpolation_names():
    assert _check_interpolation("default") == "linear"
    assert _check_interpolation("nearest") == "nearest"
    with pytest.raises(BadInput):
        _check_interpolation("spline")


def test_conductivity_lookup_takes_the_upper_element_and_none_at_the_last_node():
    """ThermalConductivityData::at (therm3d.cpp:421-435): findUpIndex - 1 per axis, NaN
    when findUpIndex is 0 or the axis size."""
    a = np.array([0.0, 1.0, 3.0, 4.0])
    pts = np.array([[-0.5], [0.0], [0.5], [1.0], [3.9], [4.0], [5.0]])
    idx, ok = conductivity_elements((a,), pts)
    assert ok.tolist() == [False, True, True, True, True, False, False]
    assert idx[0][ok].tolist() == [0, 0, 1, 2]


def test_full_mesh_interpolation_continues_the_edge_values_outside():
    """prepareInterpolationForAxis (plask/mesh/axis1d.cpp:99-154) gives both bracketing
    nodes the edge index outside an axis, so a full mesh's linear interpolation returns
    the edge values there (no NaN for the solver's SafeData to replace)."""
    from plask_gb300.thermal import _trilinear
    from plask_gb300.thermal2d import _bilinear

    ax = (np.array([0.0, 1.0, 2.0]), np.array([0.0, 2.0]), np.array([0.0, 1.0]))
    F = np.arange(12, dtype=float).reshape(2, 2, 3)
    pts = np.array([[-5.0, 1.0, 0.5], [9.0, 1.0, 0.5], [0.5, -1.0, 3.0]])
    out = _trilinear(ax, F, pts, fill=None)
    inside = _trilinear(ax, F, np.array([[0.0, 1.0, 0.5], [2.0, 1.0, 0.5], [0.5, 0.0, 1.0]]), fill=None)
    np.testing.assert_allclose(out, inside)
    G = F[0]
    out2 = _bilinear(ax[:2], G, np.array([[-1.0, 0.5], [3.0, 5.0]]), fill=None)
    np.testing.assert_allclose(out2, _bilinear(ax[:2], G, np.array([[0.0, 0.5], [2.0, 2.0]]), fill=None))


def test_boundary_condition_list_interface():
    """python/plask/python/boundaries.hpp:53-160: append, prepend, insert, negative indices,
    tuple assignment, deletion, clear."""
    from plask_gb300 import thermal as TH

    sv = TH.Static3D()
    bc = sv.convection_boundary
    bc.append("top", {"coeff": 10.0, "ambient": 300.0})
    bc.prepend("bottom", (5.0, 290.0))
    bc.insert(1, "left", {"coeff": 1.0, "ambient": 280.0})
    assert [p for p, _ in bc] == ["bottom", "left", "top"]
    assert bc[-1] == ("top", (10.0, 300.0))
    bc[0] = ("front", {"coeff": 2.0, "ambient": 310.0})
    assert bc[0] == ("front", (2.0, 310.0))
    with pytest.raises(TypeError):
        bc[0] = "front"
    with pytest.raises(IndexError):
        bc[5]
    del bc[-1]
    assert len(bc) == 2 and "front" in repr(bc)
    bc.clear()
    assert len(bc) == 0
