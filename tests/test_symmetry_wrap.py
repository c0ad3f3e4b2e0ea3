"""Mirrored coordinates of the providers (InterpolationFlags::wrap / postprocess,
plask/mesh/interpolation.hpp:232-287) for geometries on either side of the mirror."""
import numpy as np

from plask_gb300.mesh import wrap_symmetric


def test_positive_side_reads_absolute_values_and_flips_negative_points():
    pts = np.array([[-2.0, 1.0, 3.0], [0.0, -1.0, 2.0], [4.0, 5.0, 6.0]])
    w, flips = wrap_symmetric(pts, (True, False, False), (0.0, -3.0, 0.0))
    assert np.array_equal(w[:, 0], [2.0, 1e-12, 4.0])
    assert np.array_equal(w[:, 1:], pts[:, 1:])
    assert list(flips) == [0] and flips[0].tolist() == [True, False, False]


def test_negative_side_reads_minus_absolute_values_and_flips_positive_points():
    pts = np.array([[-2.0, 0.0], [3.0, 0.0], [0.0, 0.0]])
    w, flips = wrap_symmetric(pts, (True, False), (-10.0, 0.0))
    assert np.array_equal(w[:, 0], [-2.0, -3.0, -1e-12])
    assert flips[0].tolist() == [False, True, False]


def test_no_symmetric_axis_leaves_points_alone():
    pts = np.array([[-1.0, 2.0, 3.0]])
    w, flips = wrap_symmetric(pts, (False, False, False), (0.0, 0.0, 0.0))
    assert w is pts and flips == {}


def test_symmetric_axis_spanning_both_sides_is_rejected():
    import pytest

    pts = np.array([[1.0, 2.0, 3.0]])
    with pytest.raises(ValueError, match="both sides of transverse axis"):
        wrap_symmetric(pts, (False, True, False), (0.0, -2.0, 0.0), (5.0, 2.0, 9.0))
    w, _ = wrap_symmetric(pts, (False, True, False), (0.0, 0.0, 0.0), (5.0, 2.0, 9.0))
    assert w[0, 1] == 2.0
