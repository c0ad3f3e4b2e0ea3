"""Providers on masked meshes (CPU): the element search and interpolation of
RectangularMaskedMesh2D/3D (plask/mesh/rectangular_masked3d.cpp:68-112,
rectangular_masked2d.cpp:58-89, rectangular_masked3d.hpp:555-603) that the thermal
providers use when empty elements are left out, with NaN read as 300 K by the solver
(SafeData, solvers/thermal/static/therm3d.cpp:387-395)."""
import numpy as np

from plask_gb300.thermal import (MASKED_MIN_DISTANCE, masked_element_interpolate, masked_element_search,
                                  masked_interpolate)

AX = (np.array([0.0, 1.0, 2.0, 4.0]), np.array([0.0, 0.5, 1.5]), np.array([10.0, 11.0, 13.0, 14.0]))


def _field(axes, coef):
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]  # canonical (axis 2, 1, 0)
    return coef[0] + sum(c * g for c, g in zip(coef[1:], grids))


def test_linear_field_is_reproduced_in_included_elements():
    active = np.ones((3, 2, 3), bool)
    active[1, 1, 2] = False
    F = _field(AX, (300.0, 2.0, -3.0, 0.5))
    rng = np.random.default_rng(1)
    pts = np.stack([rng.uniform(a[0], a[-1], 400) for a in AX], axis=1)
    elem, found = masked_element_search(AX, active, pts)
    out = masked_interpolate(AX, F, active, pts, "linear")
    want = 300.0 + 2.0 * pts[:, 0] - 3.0 * pts[:, 1] + 0.5 * pts[:, 2]
    assert np.allclose(out[found], want[found], rtol=0, atol=1e-12)
    # points inside the left-out element read NaN
    inside = (pts[:, 0] > 2.0) & (pts[:, 1] > 0.5) & (pts[:, 2] > 11.0) & (pts[:, 2] < 13.0)
    assert inside.any() and np.all(~found[inside]) and np.all(np.isnan(out[inside]))


def test_hole_element_reads_nan_although_its_corners_are_on_the_mesh():
    ax = (np.arange(4.0), np.arange(4.0), np.arange(4.0))
    active = np.ones((3, 3, 3), bool)
    active[1, 1, 1] = False  # every corner of the hole still belongs to other elements
    F = _field(ax, (1.0, 1.0, 1.0, 1.0))
    out = masked_interpolate(ax, F, active, np.array([[1.5, 1.5, 1.5], [0.5, 1.5, 1.5]]), "linear")
    assert np.isnan(out[0]) and out[1] == 1.0 + 0.5 + 1.5 + 1.5


def test_face_points_take_the_included_neighbour():
    ax = (np.arange(3.0), np.arange(2.0), np.arange(2.0))
    for act_left in (True, False):
        active = np.array([[[act_left, not act_left]]])
        F = _field(ax, (5.0, 1.0, 0.0, 0.0))
        # on the node line x = 1 and a hair to either side of it
        for x in (1.0, 1.0 - 0.5 * MASKED_MIN_DISTANCE, 1.0 + 0.5 * MASKED_MIN_DISTANCE):
            elem, found = masked_element_search(ax, active, np.array([[x, 0.5, 0.5]]))
            assert found[0] and elem[0][0] == (0 if act_left else 1)
        # a point clearly inside the left-out element
        elem, found = masked_element_search(ax, active, np.array([[1.5 if act_left else 0.5, 0.5, 0.5]]))
        assert not found[0]


def test_box_tolerance():
    active = np.ones((3, 2, 3), bool)
    eps = 0.5 * MASKED_MIN_DISTANCE
    pts = np.array([[-eps, 0.2, 12.0], [4.0 + eps, 0.2, 12.0], [-3 * eps, 0.2, 12.0], [1.0, 0.2, 14.0 + 3 * eps]])
    _, found = masked_element_search(AX, active, pts)
    assert found.tolist() == [True, True, False, False]


def test_nearest_corner_of_the_holding_element_lower_on_a_tie():
    ax = (np.array([0.0, 2.0, 4.0]), np.array([0.0, 1.0]))
    active = np.array([[True, False]])
    F = np.array([[1.0, 2.0, 3.0], [10.0, 20.0, 30.0]])
    pts = np.array([[1.0, 0.5], [1.2, 0.2], [0.9, 0.7], [3.0, 0.5], [2.0, 0.5]])
    out = masked_interpolate(ax, F, active, pts, "nearest")
    # ties go to the lower node; x = 2 lies on the face of the included element
    assert out[0] == 1.0 and out[1] == 2.0 and out[2] == 10.0 and np.isnan(out[3]) and out[4] == 2.0


def test_upper_neighbour_along_axis_2_compares_with_axis_1():
    """rectangular_masked3d.cpp:107 compares the third coordinate with the upper node of
    axis 1: a point a hair below a z node line does not find an included element above
    it when z exceeds that y coordinate."""
    ax_low_z = (np.arange(2.0), np.array([0.0, 5.0]), np.array([0.0, 1.0, 2.0]))
    ax_high_z = (np.arange(2.0), np.array([0.0, 0.5]), np.array([0.0, 1.0, 2.0]))
    active = np.array([[[False]], [[True]]])  # the lower element left out, the upper one included
    z = 1.0 - 0.5 * MASKED_MIN_DISTANCE
    _, found_low = masked_element_search(ax_low_z, active, np.array([[0.5, 0.2, z]]))
    _, found_high = masked_element_search(ax_high_z, active, np.array([[0.5, 0.2, z]]))
    assert found_low[0] and not found_high[0]


def _element_field(axes, coef):
    mids = [0.5 * (a[1:] + a[:-1]) for a in axes]
    return _field(mids, coef)


def test_element_values_linear_between_midpoints_with_left_out_diagonals():
    """A linear field over the midpoints is reproduced where the point lies between included
    midpoints; a left-out diagonal neighbour takes the sum of the axis neighbours less the
    holding value, which is exact for a linear field."""
    ax = (np.arange(5.0), np.arange(4.0) * 2.0, np.arange(4.0) * 0.5)
    active = np.ones((3, 3, 4), bool)
    active[2, 2, 3] = False  # a diagonal neighbour of the element (2, 1, 1) for points toward it
    Q = _element_field(ax, (1.0, 0.3, -0.2, 4.0))
    pts = np.array([[2.8, 3.4, 0.9], [1.6, 2.5, 0.3], [2.6, 3.8, 1.1]])
    out = masked_element_interpolate(ax, Q, active, pts, "linear")
    want = 1.0 + 0.3 * pts[:, 0] - 0.2 * pts[:, 1] + 4.0 * pts[:, 2]
    assert np.allclose(out, want, rtol=0, atol=1e-12)


def test_element_values_left_out_axis_neighbour_and_edges_hold_the_element_value():
    ax = (np.arange(4.0), np.arange(2.0))
    active = np.array([[True, True, False]])
    Q = np.array([[10.0, 20.0, 99.0]])
    pts = np.array([[1.8, 0.5], [0.2, 0.5], [1.2, 0.5], [2.5, 0.5]])
    out = masked_element_interpolate(ax, Q, active, pts, "linear")
    # toward the left-out element: the holding value; below the first midpoint: the edge value;
    # between the included midpoints 0.5 and 1.5: linear; inside the left-out element: NaN
    assert out[0] == 20.0 and out[1] == 10.0 and np.isclose(out[2], 10.0 + 10.0 * 0.7) and np.isnan(out[3])
    near = masked_element_interpolate(ax, Q, active, pts, "nearest")
    assert near[0] == 20.0 and near[1] == 10.0 and near[2] == 20.0 and np.isnan(near[3])


def test_element_values_with_components():
    ax = (np.arange(3.0), np.arange(3.0))
    active = np.array([[True, True], [True, False]])
    Q = np.stack([_element_field(ax, (0.0, 1.0, 0.0)), _element_field(ax, (0.0, 0.0, 1.0))], axis=-1)
    out = masked_element_interpolate(ax, Q, active, np.array([[0.9, 0.7], [1.5, 1.5]]), "linear")
    assert np.allclose(out[0], [0.9, 0.7]) and np.all(np.isnan(out[1]))


def test_electrical_voltage_provider_on_the_masked_diode():
    """Shockley3D.outVoltage on the reference diode's masked mesh (air left out), with the
    potential read from a stand-in for the device handle: NaN in the air, the trilinear
    value of the holding element in the conductors (electr3d.cpp:507-515)."""
    from plask_gb300 import electrical as EL
    from plask_gb300 import structures as S

    s = S.shockley_diode()
    sv = EL.solver_for_structure(s, ordering="012", algorithm="gpu-mixed")

    class _Handle:
        @staticmethod
        def potential(nn):
            return np.linspace(0.0, 1.0, nn)

    sv._elec = _Handle()
    V = sv._full_potential()
    x, y, z = s.axes
    air = np.array([[480.0, 480.0, 0.5]])          # in the bottom contact layer, beside the contact: air
    metal = np.array([[0.0, 0.0, 450.0]])           # inside the upper conductor block
    assert np.isnan(sv.outVoltage(air)[0])
    got = sv.outVoltage(metal)[0]
    i = [np.searchsorted(a, p, side="right") - 1 for a, p in zip(s.axes, metal[0])]
    w = [(metal[0][d] - s.axes[d][i[d]]) / (s.axes[d][i[d] + 1] - s.axes[d][i[d]]) for d in range(3)]
    want = sum((w[0] if a else 1 - w[0]) * (w[1] if b else 1 - w[1]) * (w[2] if c else 1 - w[2])
               * V[i[2] + c, i[1] + b, i[0] + a] for a in (0, 1) for b in (0, 1) for c in (0, 1))
    assert np.isfinite(got) and np.isclose(got, want, rtol=0, atol=1e-12)


def test_thermal_temperature_provider_on_a_masked_mesa():
    """Static3D.outTemperature on an etched mesa (a masked mesh), the temperatures read from a
    stand-in for the device handle: 300 K where no included element holds the point
    (SafeData, therm3d.cpp:387-395), the holding element's trilinear value elsewhere; the
    spline method through the same path."""
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    s = S.layered_c0(seed=2, n=(8, 8, 12), power=1e15)
    n_mat = s.k300.size
    s.k300, s.p = np.append(s.k300, 0.026), np.append(s.p, 0.0)
    s.kz_ratio, s.hexp, s.empty = np.append(s.kz_ratio, 1.0), np.append(s.hexp, 0.0), np.append(s.empty, True)
    xm = 0.5 * (s.axes[0][1:] + s.axes[0][:-1])
    mat = s.mat.copy()
    mat[-3:, :, xm > 10.0] = n_mat  # the top three element layers etched away beyond x = 10 um
    s.mat = mat
    sv = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    nn = int(sv._active_mask_mesh_order().sum())

    class _Handle:
        @staticmethod
        def temperature():
            return np.linspace(300.0, 400.0, nn)

        @staticmethod
        def sizes():
            return nn, 0

    sv._fem = _Handle()
    T = sv._full_temperature()
    z = s.axes[2]
    etched = np.array([[40.0, 5.0, 0.5 * (z[-1] + z[-2])]])
    inside = np.array([[2.0, 3.0, 0.5 * (z[-1] + z[-2])]])
    assert sv.outTemperature(etched)[0] == 300.0
    assert sv.outTemperature(etched, "spline")[0] == 300.0
    got = sv.outTemperature(inside)[0]
    assert np.isfinite(got) and T[np.isfinite(T)].min() <= got <= T[np.isfinite(T)].max()
    # outside the mesh box a masked mesh has no element: 300 K
    assert sv.outTemperature(np.array([[-5.0, 3.0, 1.0]]))[0] == 300.0


def _search_by_loops(axes, active, p):
    """The nested loops of RectangularMaskedMesh3D::prepareInterpolation
    (rectangular_masked3d.cpp:68-112), one point at a time."""
    MIN = MASKED_MIN_DISTANCE
    if not all(a[0] - x < MIN and x - a[-1] < MIN for a, x in zip(axes, p)):
        return None
    lo, hi = [], []
    for a, x in zip(axes, p):
        h = int(np.searchsorted(a, x, side="right"))
        h = a.size - 1 if h == a.size else (1 if h == 0 else h)
        lo.append(h - 1)
        hi.append(h)
    lo_c = [a[i] for a, i in zip(axes, lo)]
    hi_c = [a[i] for a, i in zip(axes, hi)]
    i0, i1, i2 = lo
    for _ in range(2):
        for _ in range(2):
            for _ in range(2):
                if active[i2, i1, i0]:
                    return (i0, i1, i2)
                if i0 > 0 and lo_c[0] <= p[0] < lo_c[0] + MIN:
                    i0 = hi[0] - 2
                elif i0 < axes[0].size - 2 and hi_c[0] - MIN < p[0] <= hi_c[0]:
                    i0 = hi[0]
                else:
                    break
            i0 = hi[0] - 1
            if i1 > 0 and lo_c[1] <= p[1] < lo_c[1] + MIN:
                i1 = hi[1] - 2
            elif i1 < axes[1].size - 2 and hi_c[1] - MIN < p[1] <= hi_c[1]:
                i1 = hi[1]
            else:
                break
        i1 = hi[1] - 1
        if i2 > 0 and lo_c[2] <= p[2] < lo_c[2] + MIN:
            i2 = hi[2] - 2
        elif i2 < axes[2].size - 2 and hi_c[2] - MIN < p[2] <= hi_c[1]:
            i2 = hi[2]
        else:
            break
    return None


def test_vectorised_search_matches_the_reference_loops():
    rng = np.random.default_rng(11)
    axes = (np.array([0.0, 1.0, 2.0, 3.5]), np.array([0.0, 0.8, 3.0, 3.2]), np.array([0.0, 2.0, 2.5, 4.0]))
    for trial in range(20):
        active = rng.random((3, 3, 3)) < 0.5
        # points on and within the tolerance of node lines, inside elements and just outside the box
        pts = []
        for _ in range(150):
            p = []
            for a in axes:
                kind = rng.integers(4)
                node = a[rng.integers(a.size)]
                if kind == 0:
                    p.append(node)
                elif kind == 1:
                    p.append(node + rng.choice([-0.5, 0.5]) * MASKED_MIN_DISTANCE)
                elif kind == 2:
                    p.append(rng.uniform(a[0], a[-1]))
                else:
                    p.append(node + rng.choice([-3.0, 3.0]) * MASKED_MIN_DISTANCE)
            pts.append(p)
        pts = np.array(pts)
        elem, found = masked_element_search(axes, active, pts)
        for k, p in enumerate(pts):
            want = _search_by_loops(axes, active, p)
            if want is None:
                assert not found[k], (trial, p)
            else:
                assert found[k] and (elem[0][k], elem[1][k], elem[2][k]) == want, (trial, p, want)


def _element_linear_by_loops(axes, Q, active, p):
    """RectangularMaskedMesh3D::ElementMesh::interpolateLinear (rectangular_masked3d.hpp:277-333)."""
    hit = _search_by_loops(axes, active, p)
    if hit is None:
        return np.nan
    i0, i1, i2 = hit
    mids = [0.5 * (a[1:] + a[:-1]) for a in axes]
    pa = [mids[0][i0], mids[1][i1], mids[2][i2]]

    def step(d, i):
        if p[d] < pa[d]:
            return 0 if i == 0 else -1
        return 0 if i + 1 == mids[d].size else 1

    s0, s1, s2 = step(0, i0), step(1, i1), step(2, i2)

    def val(a, b, c):
        return Q[c, b, a] if active[c, b, a] else None

    aaa = Q[i2, i1, i0]
    if s0 == 0 and s1 == 0 and s2 == 0:
        return aaa
    aab = val(i0, i1, i2 + s2)
    aba = val(i0, i1 + s1, i2)
    baa = val(i0 + s0, i1, i2)
    aab = aaa if aab is None else aab
    aba = aaa if aba is None else aba
    baa = aaa if baa is None else baa
    abb = val(i0, i1 + s1, i2 + s2)
    bab = val(i0 + s0, i1, i2 + s2)
    bba = val(i0 + s0, i1 + s1, i2)
    bbb = val(i0 + s0, i1 + s1, i2 + s2)
    abb = aab + aba - aaa if abb is None else abb
    bab = baa + aab - aaa if bab is None else bab
    bba = aba + baa - aaa if bba is None else bba
    bbb = aab + aba + baa - 2 * aaa if bbb is None else bbb
    pb = [mids[0][i0 + s0] + (s0 == 0), mids[1][i1 + s1] + (s1 == 0), mids[2][i2 + s2] + (s2 == 0)]
    t = [(p[d] - pa[d]) / (pb[d] - pa[d]) for d in range(3)]
    corners = {(0, 0, 0): aaa, (1, 0, 0): baa, (0, 1, 0): aba, (0, 0, 1): aab,
               (1, 1, 0): bba, (1, 0, 1): bab, (0, 1, 1): abb, (1, 1, 1): bbb}
    return sum(v * (t[0] if c[0] else 1 - t[0]) * (t[1] if c[1] else 1 - t[1]) * (t[2] if c[2] else 1 - t[2])
               for c, v in corners.items())


def test_vectorised_element_interpolation_matches_the_reference_loops():
    rng = np.random.default_rng(12)
    axes = (np.array([0.0, 1.0, 2.0, 3.5, 4.0]), np.array([0.0, 0.8, 3.0, 3.2]), np.array([0.0, 2.0, 2.5, 4.0]))
    for trial in range(10):
        active = rng.random((3, 3, 4)) < 0.6
        Q = rng.normal(size=(3, 3, 4))
        pts = np.stack([rng.uniform(a[0], a[-1], 300) for a in axes], axis=1)
        out = masked_element_interpolate(axes, Q, active, pts, "linear")
        want = np.array([_element_linear_by_loops(axes, Q, active, p) for p in pts])
        assert np.array_equal(np.isnan(out), np.isnan(want))
        ok = ~np.isnan(want)
        np.testing.assert_allclose(out[ok], want[ok], rtol=0, atol=1e-12)


def test_cylindrical_providers_mirror_negative_radii():
    """The cylindrical geometry is symmetric in r (plask/geometry/space.hpp:1068-1072): a
    StaticCyl provider reads r < 0 at |r| (InterpolationFlags::wrap)."""
    from plask_gb300 import structures as S
    from plask_gb300 import thermal2d as T2

    s = S.layered_2d(seed=5, n=(12, 14))
    sv = T2.solver_for_structure2d(s, cls=T2.StaticCyl, ordering="10")
    n = len(sv.mesh)

    class _Handle:
        @staticmethod
        def temperature():
            return 300.0 + np.arange(n, dtype=float) % 17

        @staticmethod
        def sizes():
            return n, 0

    sv._fem = _Handle()
    z = 0.5 * (s.axes[1][3] + s.axes[1][4])
    pts = np.array([[7.3, z], [-7.3, z], [0.0, z]])
    for m in ("linear", "nearest", "spline"):
        out = sv.outTemperature(pts, m)
        assert out[0] == out[1]
    w, flips = sv._wrap(pts)
    assert flips[0].tolist() == [False, True, False] and w[1, 0] == 7.3 and w[2, 0] == 1e-12
    flat = T2.solver_for_structure2d(s, cls=T2.Static2D, ordering="10")
    assert flat._wrap(pts)[1] == {}


def test_electrical_providers_mirror_the_symmetric_axes():
    """The quarter-device structure (symmetric in axes 0 and 1): the voltage at (-x, -y) is
    the one at (x, y) and the current density's x and y components change sign."""
    from plask_gb300 import electrical as EL
    from plask_gb300 import structures as S

    s = S.shockley_c4(seed=4001, n=(9, 8, 10), voltage=1.9)
    sv = EL.solver_for_structure(s, ordering="012", algorithm="gpu-mixed")
    n = len(sv.mesh)

    class _Handle:
        @staticmethod
        def potential(nn):
            return np.linspace(0.0, 1.9, nn)

    sv._elec = _Handle()
    z = 0.5 * (s.axes[2][2] + s.axes[2][3])
    pts = np.array([[3.0, 2.0, z], [-3.0, -2.0, z], [3.0, -2.0, z]])
    v = sv.outVoltage(pts)
    assert v[0] == v[1] == v[2]
    j = np.zeros(sv.mesh.element_shape + (3,))
    j[..., 0], j[..., 1], j[..., 2] = 1.0, 2.0, 3.0
    out = sv._element_interp(j, pts=pts)
    np.testing.assert_allclose(out, [[1.0, 2.0, 3.0], [-1.0, -2.0, 3.0], [1.0, -2.0, 3.0]])


def test_symmetric_thermal_geometry_mirrors_the_providers():
    """A Static3D geometry mirrored at x = 0 and y = 0 (PLaSK's mirror edges): the temperature
    at (-x, -y) is the one at (x, y)."""
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    s = S.layered_c0(seed=2, n=(7, 6, 9), power=1e15)
    sv = TH.solver_for_structure(s, ordering="012", algorithm="gpu-mixed")
    sv.geometry = TH.StructureGeometry(sv.geometry.materials, mat=s.mat, symmetric=(True, True, False))
    n = len(sv.mesh)

    class _Handle:
        @staticmethod
        def temperature():
            return 300.0 + (np.arange(n) % 11).astype(float)

        @staticmethod
        def sizes():
            return n, 0

    sv._fem = _Handle()
    z = 0.5 * (s.axes[2][2] + s.axes[2][3])
    pts = np.array([[4.0, 6.0, z], [-4.0, -6.0, z], [4.0, -6.0, z]])
    for m in ("linear", "nearest", "smooth_spline"):
        out = sv.outTemperature(pts, m)
        assert out[0] == out[1] == out[2]
