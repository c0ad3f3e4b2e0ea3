"""Spline providers (CPU): "spline" (Hyman-filtered parabolic slopes,
plask/mesh/rectangular_spline.cpp:285-360, hyman.hpp:26-31) and "smooth_spline" (the C2
spline with zero end slopes, rectangular_spline.cpp:440-600), evaluated with the spline
formula of SplineRect2D/3DLazyDataImpl::at (rectangular_spline.cpp:30-237)."""
import numpy as np
import pytest
from scipy.interpolate import CubicSpline

from plask_gb300.thermal import BadInput, _check_interpolation, hyman_diffs, smooth_spline_diffs, spline_interpolate

AX = (np.array([0.0, 0.7, 1.5, 2.0, 3.1, 4.0]), np.array([0.0, 1.0, 1.6, 2.5, 3.0]), np.array([0.0, 0.4, 1.0, 1.3, 2.0]))


def _grid(axes):
    return np.meshgrid(*axes[::-1], indexing="ij")[::-1]  # coordinates, canonical (axis 0 last)


def test_method_names():
    assert _check_interpolation("SPLINE", splines=True) == "spline"
    assert _check_interpolation("smooth_spline", splines=True) == "smooth_spline"
    with pytest.raises(BadInput):
        _check_interpolation("fourier", splines=True)


def test_spline_reproduces_node_values_and_interior_quadratics():
    x, y, z = _grid(AX)
    F = (x - 0.5) ** 2 + 2.0 * (y + 1.0) ** 2 + 0.5 * (z + 2.0) ** 2
    # at the nodes: the node values
    nodes = np.stack([g.ravel() for g in (x, y, z)], axis=1)
    np.testing.assert_allclose(spline_interpolate(AX, F, nodes, "spline"), F.ravel(), rtol=0, atol=1e-12)
    # between interior nodes a sum of monotone quadratics is exact (the parabolic slope is exact there)
    rng = np.random.default_rng(3)
    pts = np.stack([rng.uniform(a[1], a[-2], 200) for a in AX], axis=1)
    want = (pts[:, 0] - 0.5) ** 2 + 2.0 * (pts[:, 1] + 1.0) ** 2 + 0.5 * (pts[:, 2] + 2.0) ** 2
    D = hyman_diffs(AX, F)
    exact = all(np.allclose(_interior(D[d], d), _interior(dF, d)) for d, dF in enumerate(
        (2 * (x - 0.5), 4 * (y + 1.0), 1.0 * (z + 2.0))))
    assert exact
    np.testing.assert_allclose(spline_interpolate(AX, F, pts, "spline"), want, rtol=1e-12)


def _interior(A, d):
    idx = [slice(None)] * A.ndim
    idx[A.ndim - 1 - d] = slice(1, -1)
    return A[tuple(idx)]


def test_hyman_filter_keeps_a_step_monotone():
    a = (np.linspace(0.0, 5.0, 6), np.array([0.0, 1.0]))
    F = np.tile(np.array([0.0, 0.0, 0.0, 1.0, 1.0, 1.0]), (2, 1))
    xs = np.linspace(0.0, 5.0, 101)
    out = spline_interpolate(a, F, np.stack([xs, np.full_like(xs, 0.5)], axis=1), "spline")
    assert np.all(np.diff(out) >= -1e-15) and out.min() >= -1e-15 and out.max() <= 1.0 + 1e-15


def test_smooth_spline_is_the_clamped_cubic_spline():
    x, y, z = _grid(AX)
    g = np.sin(x) + 0.3 * x ** 3
    F = g + 0.0 * y + 0.0 * z
    cs = CubicSpline(AX[0], np.sin(AX[0]) + 0.3 * AX[0] ** 3, bc_type="clamped")
    xs = np.linspace(0.0, 4.0, 77)
    pts = np.stack([xs, np.full_like(xs, 1.3), np.full_like(xs, 0.9)], axis=1)
    np.testing.assert_allclose(spline_interpolate(AX, F, pts, "smooth_spline"), cs(xs), rtol=0, atol=1e-12)
    S = smooth_spline_diffs(AX, F)
    np.testing.assert_allclose(S[0][0, 0], cs(AX[0], 1), rtol=0, atol=1e-12)
    assert np.all(S[1] == 0.0) and np.all(S[2] == 0.0)


def test_outside_the_mesh_the_edge_values_continue():
    x, y, z = _grid(AX)
    F = x + 2 * y + 3 * z
    pts = np.array([[-1.0, 1.0, 1.0], [9.0, 1.0, 1.0]])
    edge = np.array([[0.0, 1.0, 1.0], [4.0, 1.0, 1.0]])
    for m in ("spline", "smooth_spline"):
        np.testing.assert_allclose(spline_interpolate(AX, F, pts, m), spline_interpolate(AX, F, edge, m), atol=1e-12)


def test_masked_spline():
    ax = (np.arange(4.0), np.arange(3.0))
    active = np.array([[True, True, False], [True, True, True]])
    x, y = _grid(ax)
    F = x + y
    F[0, 3] = np.nan  # the node only the left-out element touches
    out = spline_interpolate(ax, F, np.array([[2.5, 0.5], [1.5, 0.5], [2.5, 1.5]]), "spline", active)
    assert np.isnan(out[0]) and np.isfinite(out[1:]).all()
    with pytest.raises(BadInput):
        spline_interpolate(ax, F, np.array([[1.5, 0.5]]), "smooth_spline", active)
