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


def test_spline_formula_matches_a_transcription_of_the_reference():
    """SplineRect3DLazyDataImpl::at (rectangular_spline.cpp:102-237, no symmetry) written out
    term by term for random data, against the vectorised evaluation."""
    from plask_gb300.thermal import _hermite

    rng = np.random.default_rng(4)
    F = rng.normal(size=(AX[2].size, AX[1].size, AX[0].size))
    D0, D1, D2 = hyman_diffs(AX, F)
    pts = np.stack([rng.uniform(a[0] - 0.5, a[-1] + 0.5, 60) for a in AX], axis=1)
    got = spline_interpolate(AX, F, pts, "spline")
    for k, p in enumerate(pts):
        idx, bounds = [], []
        for a, x in zip(AX, p):
            up = int(np.searchsorted(a, x, side="right"))
            lo = 0 if up == 0 else up - 1
            lo_c = a[0] - 1.0 if up == 0 else a[up - 1]
            hi = a.size - 1 if up == a.size else up
            hi_c = a[-1] + 1.0 if up == a.size else a[up]
            idx.append((lo, hi))
            bounds.append((lo_c, hi_c))
        (l0, h0), (l1, h1), (l2, h2) = idx
        d = [b[1] - b[0] for b in bounds]
        x = [(p[i] - bounds[i][0]) / d[i] for i in range(3)]
        (h0l, h0h, g0l, g0h), (h1l, h1h, g1l, g1h), (h2l, h2h, g2l, g2h) = (_hermite(x[i], d[i]) for i in range(3))

        def f(a, b, c, A=F):
            return A[c, b, a]

        D_ll = g0l * f(l0, l1, l2, D0) + g0h * f(h0, l1, l2, D0)
        Dl_l = g1l * f(l0, l1, l2, D1) + g1h * f(l0, h1, l2, D1)
        Dll_ = g2l * f(l0, l1, l2, D2) + g2h * f(l0, l1, h2, D2)
        D_lh = g0l * f(l0, l1, h2, D0) + g0h * f(h0, l1, h2, D0)
        Dl_h = g1l * f(l0, l1, h2, D1) + g1h * f(l0, h1, h2, D1)
        Dlh_ = g2l * f(l0, h1, l2, D2) + g2h * f(l0, h1, h2, D2)
        D_hl = g0l * f(l0, h1, l2, D0) + g0h * f(h0, h1, l2, D0)
        Dh_l = g1l * f(h0, l1, l2, D1) + g1h * f(h0, h1, l2, D1)
        Dhl_ = g2l * f(h0, l1, l2, D2) + g2h * f(h0, l1, h2, D2)
        D_hh = g0l * f(l0, h1, h2, D0) + g0h * f(h0, h1, h2, D0)
        Dh_h = g1l * f(h0, l1, h2, D1) + g1h * f(h0, h1, h2, D1)
        Dhh_ = g2l * f(h0, h1, l2, D2) + g2h * f(h0, h1, h2, D2)
        want = (h0l * h1l * h2l * f(l0, l1, l2) + h0l * h1l * h2h * f(l0, l1, h2) + h0l * h1h * h2l * f(l0, h1, l2)
                + h0l * h1h * h2h * f(l0, h1, h2) + h0h * h1l * h2l * f(h0, l1, l2) + h0h * h1l * h2h * f(h0, l1, h2)
                + h0h * h1h * h2l * f(h0, h1, l2) + h0h * h1h * h2h * f(h0, h1, h2)
                + h1l * h2l * D_ll + h0l * h2l * Dl_l + h0l * h1l * Dll_
                + h1l * h2h * D_lh + h0l * h2h * Dl_h + h0l * h1h * Dlh_
                + h1h * h2l * D_hl + h0h * h2l * Dh_l + h0h * h1l * Dhl_
                + h1h * h2h * D_hh + h0h * h2h * Dh_h + h0h * h1h * Dhh_)
        assert abs(got[k] - want) <= 1e-12 * max(1.0, abs(want)), (k, got[k], want)


def test_masked_hyman_slopes_match_a_transcription_of_the_reference():
    """masked_hyman::computeDiffs (rectangular_masked_spline.cpp:436-500, no symmetry): 0 at
    the ends and next to a node off the mesh, else the limited parabolic estimate."""
    rng = np.random.default_rng(8)
    a = np.cumsum(rng.uniform(0.2, 1.5, 9))
    for _ in range(30):
        y = rng.normal(size=a.size)
        y[rng.random(a.size) < 0.25] = np.nan
        want = np.zeros(a.size)
        for i in range(1, a.size - 1):
            if np.isnan(y[i]):
                continue
            if np.isnan(y[i - 1]) or np.isnan(y[i + 1]):
                continue
            da, db = a[i] - a[i - 1], a[i + 1] - a[i]
            sa, sb = (y[i] - y[i - 1]) / da, (y[i + 1] - y[i]) / db
            v = (da * sb + db * sa) / (da + db)
            lim = 3 * min(abs(sa), abs(sb))
            want[i] = lim if v > lim else (-lim if v < -lim else v)
        got = hyman_diffs((a,), y)[0]
        ok = ~np.isnan(y)
        np.testing.assert_allclose(got[ok], want[ok], rtol=0, atol=1e-14)
