"""``Static3D``: the 3D finite-element thermal solver, on the GPU.

A drop-in for PLaSK's ``thermal.static.Static3D``
(solvers/thermal/static/therm3d.hpp:27-139, python/therm_python.cpp:136-151,
plask/common/fem/python.hpp:31-41): the same attribute names, defaults,
boundary-condition lists, receiver and providers.  The computation runs in
``libplgpu_fem3d.so``; this module only converts between PLaSK-style inputs
and the library's arrays.

Geometry: PLaSK asks its geometry tree for the material at every element
midpoint.  Here ``geometry`` is any object with ``materials`` (a
:class:`MaterialTable`) and ``material_ids(mesh)`` returning one material id
per element (canonical shape), e.g. :class:`StructureGeometry`.
"""
from __future__ import annotations

import dataclasses
import itertools
import logging

import numpy as np

from . import _native
from .mesh import RectangularMesh3D, to_mesh_order, wrap_symmetric

log = logging.getLogger("plask_gb300.thermal")

ComputationError = _native.ComputationError
BadInput = _native.BadInput


@dataclasses.dataclass
class MaterialTable:
    """Materials of a structure: k_xy(T, h) = k300 (300/T)^p h^hexp, k_z = kz_ratio k_xy."""

    k300: np.ndarray
    p: np.ndarray
    kz_ratio: np.ndarray | None = None
    hexp: np.ndarray | None = None
    empty: np.ndarray | None = None
    cp: np.ndarray | None = None     # heat capacity J/(kg K), for Dynamic3D
    dens: np.ndarray | None = None   # density kg/m^3, for Dynamic3D
    # tabulated k(T) replacing the power law of some materials: {material id: (T, k_xy, k_z or None)},
    # linear in T between the points, constant beyond the ends (the h**hexp factor still applies)
    tables: dict | None = None

    def __post_init__(self):
        self.k300 = np.asarray(self.k300, np.float64)
        n = self.k300.size
        self.p = np.asarray(self.p, np.float64)
        self.kz_ratio = np.ones(n) if self.kz_ratio is None else np.asarray(self.kz_ratio, np.float64)
        self.hexp = np.zeros(n) if self.hexp is None else np.asarray(self.hexp, np.float64)
        self.empty = np.zeros(n, bool) if self.empty is None else np.asarray(self.empty, bool)

    def tabulate(self, m, thermk, T):
        """Replace material m's power law by a table sampled from ``thermk(T) -> (k_xy, k_z)``
        (the way a caller binds a material's Material::thermk, plask/material/material.hpp:691)
        at the strictly increasing temperatures T."""
        T = np.asarray(T, np.float64)
        kxy, kz = zip(*(thermk(float(t)) for t in T))
        if self.tables is None:
            self.tables = {}
        self.tables[int(m)] = (T, np.asarray(kxy, np.float64), np.asarray(kz, np.float64))

    def thermk(self, m, T, h=None):
        m = np.asarray(m)
        kxy = self.k300[m] * (300.0 / np.asarray(T)) ** self.p[m]
        if h is not None and np.any(self.hexp[m] != 0):
            kxy = kxy * np.asarray(h) ** self.hexp[m]
        kz = kxy * self.kz_ratio[m]
        if self.tables:
            Tb = np.broadcast_to(np.asarray(T, np.float64), m.shape)
            kxy, kz = np.array(kxy, np.float64, copy=True), np.array(kz, np.float64, copy=True)
            for mid, tab in self.tables.items():
                sel = m == mid
                if not np.any(sel):
                    continue
                t, a = np.asarray(tab[0], np.float64), np.asarray(tab[1], np.float64)
                c = a if len(tab) < 3 or tab[2] is None else np.asarray(tab[2], np.float64)
                ka, kc = np.interp(Tb[sel], t, a), np.interp(Tb[sel], t, c)
                if h is not None and self.hexp[mid] != 0:
                    f = np.broadcast_to(np.asarray(h, np.float64), m.shape)[sel] ** self.hexp[mid]
                    ka, kc = ka * f, kc * f
                kxy[sel], kz[sel] = ka, kc
        return kxy, kz

    def apply_tables(self, fem):
        """Send the tables to a native handle (after its set_materials)."""
        for mid, tab in (self.tables or {}).items():
            fem.set_material_table(int(mid), tab[0], tab[1], None if len(tab) < 3 else tab[2])


class StructureGeometry:
    """Geometry given directly as element material ids on a fixed mesh (or a callable of midpoints).

    ``symmetric``: per axis, whether the geometry is mirrored at 0 (a ``mirror`` edge in
    PLaSK, plask/geometry/space.hpp:147-150); the providers then read negative coordinates
    at their absolute values."""

    def __init__(self, materials: MaterialTable, mat=None, material_at=None, leaf_height=None,
                 symmetric=(False, False, False)):
        self.materials = materials
        self._mat = None if mat is None else np.asarray(mat, np.int32)
        self._at = material_at
        self._leaf = leaf_height
        self.symmetric = tuple(bool(v) for v in symmetric)

    def material_ids(self, mesh: RectangularMesh3D):
        if self._mat is not None:
            if self._mat.shape != mesh.element_shape:
                raise BadInput(-1, f"material ids of shape {self._mat.shape} do not fit the mesh {mesh.element_shape}")
            return self._mat
        if self._at is None:
            raise BadInput(-1, "geometry has neither material ids nor a material function")
        mids = mesh.element_midpoints()
        return np.asarray(self._at(mids[..., 0], mids[..., 1], mids[..., 2]), np.int32)

    def leaf_height(self, mesh):
        return None if self._leaf is None else np.asarray(self._leaf, np.float64)

    @classmethod
    def from_structure(cls, s):
        return cls(MaterialTable(s.k300, s.p, s.kz_ratio, s.hexp, s.empty, tables=getattr(s, "ktables", None)),
                   mat=s.mat)


class BoundaryConditions:
    """Ordered list of (place, value) pairs (BoundaryConditions, boundary_conditions.hpp;
    the Python interface of python/plask/python/boundaries.hpp:53-160: indexing from the end
    with negative numbers, assignment of a (place, value) tuple, append, prepend, insert,
    clear, deletion, iteration)."""

    def __init__(self, owner, kind, nvals):
        self._owner = owner
        self._kind = kind
        self._nvals = nvals
        self._items = []

    def _norm(self, value):
        if self._nvals == 1:
            return (float(value),)
        if isinstance(value, dict):
            keys = ("coeff", "ambient") if self._kind == _native.BC_CONVECTION else ("emissivity", "ambient")
            return tuple(float(value[k]) for k in keys)
        return tuple(float(v) for v in value)

    def append(self, place, value):
        self._items.append((place, self._norm(value)))
        self._owner._bc_changed()

    def prepend(self, place, value):
        self._items.insert(0, (place, self._norm(value)))
        self._owner._bc_changed()

    def insert(self, index, place, value):
        self._items.insert(index, (place, self._norm(value)))
        self._owner._bc_changed()

    def _index(self, i):
        j = i + len(self._items) if i < 0 else i
        if not 0 <= j < len(self._items):
            raise IndexError("boundary conditions index out of range")
        return j

    def __setitem__(self, i, item):
        try:
            place, value = item
        except (TypeError, ValueError):
            raise TypeError("you can only assign a tuple (boundary, value)") from None
        self._items[self._index(i)] = (place, self._norm(value))
        self._owner._bc_changed()

    def clear(self):
        self._items.clear()
        self._owner._bc_changed()

    def __delitem__(self, i):
        del self._items[i]
        self._owner._bc_changed()

    def __getitem__(self, i):
        return self._items[self._index(i)]

    def __repr__(self):
        return "[" + ", ".join(f"({p!r}, {v[0] if len(v) == 1 else v})" for p, v in self._items) + "]"

    def __len__(self):
        return len(self._items)

    def __iter__(self):
        return iter(self._items)


@dataclasses.dataclass
class IterativeParams:
    """``solver.iterative`` (plask/common/fem/iterative_matrix.hpp:25-94)."""

    accelerator: str = "cg"
    preconditioner: str = "ic"
    maxit: int = 1000
    maxerr: float = 1e-6
    noconv: str = "warning"
    nfact: int = 10
    ns1: int = 5
    ns2: int = 100000
    lvfill: int = 0
    ltrunc: int = 0
    ndeg: int = 1
    omega: float = 1.0
    converged: bool = True
    iters: int = 0
    err: float = 0.0


class Receiver:
    """``inHeat``: heat density [W/m^3]; a constant, an element array, or a callable of midpoints."""

    def __init__(self, owner, default=0.0):
        self._owner = owner
        self._value = default

    def attach(self, value):
        self._value = value
        self._owner._heat_changed()

    def __call__(self, mesh: RectangularMesh3D):
        v = self._value
        if hasattr(v, "__call__") and not isinstance(v, np.ndarray):
            mids = mesh.element_midpoints()
            return np.broadcast_to(np.asarray(v(mids[..., 0], mids[..., 1], mids[..., 2]), np.float64),
                                   mesh.element_shape)
        arr = np.asarray(v, np.float64)
        return np.broadcast_to(arr, mesh.element_shape)


class Provider:
    def __init__(self, fn):
        self._fn = fn

    def __call__(self, mesh=None, interpolation="linear"):
        return self._fn(mesh, interpolation)


def _nearest_axis(axis, x):
    """Index of the nearest node, the lower one on a tie (find_nearest_binary,
    plask/utils/stl.hpp:59-80)."""
    lb = np.searchsorted(axis, x, side="left")
    hi = np.minimum(lb, axis.size - 1)
    lo = np.maximum(lb - 1, 0)
    take_lo = (lb == axis.size) | ((lb > 0) & (x - axis[lo] <= axis[hi] - x))
    return np.where(take_lo, lo, hi)


# boundary tolerance of the masked meshes, um (plask/mesh/rectangular_masked_common.hpp:36)
MASKED_MIN_DISTANCE = 1e-9


def masked_element_search(axes, active, pts):
    """The element of a masked mesh that holds each point, found as
    RectangularMaskedMesh3D::prepareInterpolation finds it (rectangular_masked3d.cpp:68-112;
    2D: rectangular_masked2d.cpp:58-89): the element around the point (the upper one when
    the point lies on a node line) or, for a point within 1e-9 um of that element's
    faces, the neighbour across the face, tried with axis 0 varying fastest.

    ``axes``: the node axes; ``active``: canonical element mask (axis 0 last);
    ``pts``: (m, len(axes)).  Returns the low node index of the element per axis and a
    mask of the points that an included element holds (the others read NaN in the
    reference).  The reference compares the third coordinate with the upper node of
    axis 1 when it looks for the upper neighbour along axis 2 (rectangular_masked3d.cpp:107);
    that comparison is kept."""
    dims = len(axes)
    m = len(pts)
    inbox = np.ones(m, bool)
    lo, hi_c = [], []
    for d, a in enumerate(axes):
        x = pts[:, d]
        inbox &= (a[0] - x < MASKED_MIN_DISTANCE) & (x - a[-1] < MASKED_MIN_DISTANCE)
        hi = np.searchsorted(a, x, side="right")  # findUpIndex, then clamped to an element
        hi = np.where(hi >= a.size, a.size - 1, np.where(hi == 0, 1, hi))
        lo.append(hi - 1)
        hi_c.append(a[hi])
    alt, has_alt = [], []
    for d, a in enumerate(axes):
        x = pts[:, d]
        lo_c = a[lo[d]]
        upper = hi_c[1] if d == 2 else hi_c[d]
        near_lo = (lo[d] > 0) & (lo_c <= x) & (x < lo_c + MASKED_MIN_DISTANCE)
        near_hi = ~near_lo & (lo[d] < a.size - 2) & (hi_c[d] - MASKED_MIN_DISTANCE < x) & (x <= upper)
        alt.append(np.where(near_lo, lo[d] - 1, lo[d] + 1))
        has_alt.append(near_lo | near_hi)
    elem = [np.zeros(m, np.int64) for _ in range(dims)]
    found = np.zeros(m, bool)
    for tt in itertools.product((0, 1), repeat=dims):
        t = tt[::-1]  # axis 0 fastest
        valid = inbox & ~found
        for d in range(dims):
            if t[d]:
                valid &= has_alt[d]
        sel = np.flatnonzero(valid)
        if sel.size == 0:
            continue
        idx = [(alt[d] if t[d] else lo[d])[sel] for d in range(dims)]
        hit = active[tuple(idx[::-1])]
        rows = sel[hit]
        for d in range(dims):
            elem[d][rows] = idx[d][hit]
        found[rows] = True
    return elem, found


def masked_interpolate(axes, F, active, pts, method):
    """Nodal values F (canonical, NaN off the masked mesh) at points, as the masked mesh
    interpolates them (rectangular_masked3d.hpp:555-603): multilinear over the corners of
    the holding element, or its nearest corner (the lower one on a tie); NaN where no
    included element holds the point."""
    dims = len(axes)
    elem, found = masked_element_search(axes, active, pts)
    out = np.full(len(pts), np.nan)
    s = np.flatnonzero(found)
    lo = [elem[d][s] for d in range(dims)]
    x = [pts[s, d] for d in range(dims)]
    a_lo = [axes[d][lo[d]] for d in range(dims)]
    a_hi = [axes[d][lo[d] + 1] for d in range(dims)]
    if method == "nearest":
        idx = [np.where(x[d] - a_lo[d] <= a_hi[d] - x[d], lo[d], lo[d] + 1) for d in range(dims)]
        out[s] = F[tuple(idx[::-1])]
        return out
    w = [(x[d] - a_lo[d]) / (a_hi[d] - a_lo[d]) for d in range(dims)]
    val = np.zeros(s.size)
    for c in itertools.product((0, 1), repeat=dims):
        wt = np.ones(s.size)
        for d in range(dims):
            wt = wt * (w[d] if c[d] else 1.0 - w[d])
        val += wt * F[tuple((lo[d] + c[d]) for d in range(dims))[::-1]]
    out[s] = val
    return out


def masked_element_interpolate(axes, Q, active, pts, method):
    """Element values Q (canonical, components last) at points on a masked mesh, as its
    element mesh interpolates them (rectangular_masked3d.hpp:277-333,
    rectangular_masked2d.hpp:196-237): the holding element's value (nearest), or
    multilinear between its midpoint and the neighbouring midpoints on the point's side,
    a left-out neighbour along one axis taking the holding element's value and one
    along several axes the sum of the single-axis values less the holding value for
    each axis beyond the first; NaN where no included element holds the point."""
    dims = len(axes)
    elem, found = masked_element_search(axes, active, pts)
    out = np.full((len(pts),) + Q.shape[dims:], np.nan)
    s = np.flatnonzero(found)
    e = [elem[d][s] for d in range(dims)]
    if method == "nearest":
        out[s] = Q[tuple(e[::-1])]
        return out
    mids = [0.5 * (a[1:] + a[:-1]) for a in axes]
    x = [pts[s, d] for d in range(dims)]
    pa = [mids[d][e[d]] for d in range(dims)]
    step = [np.where(x[d] < pa[d], np.where(e[d] == 0, 0, -1), np.where(e[d] + 2 == axes[d].size, 0, 1))
            for d in range(dims)]
    base = Q[tuple(e[::-1])]
    corner = {(0,) * dims: base}
    # corners in order of the number of stepped axes, so that the single-axis values exist
    for c in sorted(itertools.product((0, 1), repeat=dims), key=sum):
        if sum(c) == 0:
            continue
        idx = [e[d] + c[d] * step[d] for d in range(dims)]
        inc = active[tuple(idx[::-1])]
        val = Q[tuple(idx[::-1])]
        if sum(c) == 1:
            sub = base
        else:
            singles = [corner[tuple(int(k == d) for k in range(dims))] for d in range(dims) if c[d]]
            sub = sum(singles) - (len(singles) - 1) * base
        inc = inc.reshape(inc.shape + (1,) * (base.ndim - 1))
        corner[c] = np.where(inc, val, sub)
    pb = [mids[d][e[d] + step[d]] + (step[d] == 0) for d in range(dims)]
    t = [(x[d] - pa[d]) / (pb[d] - pa[d]) for d in range(dims)]
    val = np.zeros_like(base)
    for c, v in corner.items():
        wt = np.ones(s.size)
        for d in range(dims):
            wt = wt * (t[d] if c[d] else 1.0 - t[d])
        val += wt.reshape(wt.shape + (1,) * (base.ndim - 1)) * v
    out[s] = val
    return out


def conductivity_elements(axes, pts):
    """Element of each point for the conductivity providers (ThermalConductivityData::at,
    therm3d.cpp:421-435, therm2d.cpp:581-594): findUpIndex (the first node above the
    coordinate) less one per axis, so a point on a node line takes the upper element; a
    point below the first node or on or above the last one has none.  Returns the element
    indices per axis and the mask of points that have one."""
    idx, ok = [], np.ones(len(pts), bool)
    for d, a in enumerate(axes):
        u = np.searchsorted(a, pts[:, d], side="right")
        ok &= (u > 0) & (u < a.size)
        idx.append(np.clip(u - 1, 0, a.size - 2))
    return idx, ok


def _along(F, d, sl):
    """Index F (canonical: axis 0 last) with slice ``sl`` along mesh axis d."""
    idx = [slice(None)] * F.ndim
    idx[F.ndim - 1 - d] = sl
    return F[tuple(idx)]


def _axis_shape(F, d, v):
    """v (along mesh axis d) shaped to broadcast against canonical F."""
    shp = [1] * F.ndim
    shp[F.ndim - 1 - d] = v.size
    return v.reshape(shp)


def hyman_diffs(axes, F):
    """Node derivatives along every axis for the "spline" interpolation
    (hyman::computeDiffs, plask/mesh/rectangular_spline.cpp:285-360; on a masked mesh
    masked_hyman::computeDiffs, rectangular_masked_spline.cpp:436-500), without symmetry or
    periodicity: the parabolic estimate (da sb + db sa) / (da + db) from the one-sided
    slopes sa, sb, limited to 3 min(|sa|, |sb|) (Hyman's filter, plask/mesh/hyman.hpp:26-31);
    0 at the first and last node and, on a masked mesh (NaN off it), next to a node off
    the mesh."""
    diffs = []
    for d, a in enumerate(axes):
        D = np.zeros_like(F)
        n = a.size
        if n > 2:
            Fm, F0, Fp = _along(F, d, slice(0, n - 2)), _along(F, d, slice(1, n - 1)), _along(F, d, slice(2, n))
            h = np.diff(a)
            da, db = _axis_shape(F, d, h[:-1]), _axis_shape(F, d, h[1:])
            with np.errstate(invalid="ignore"):
                sa, sb = (F0 - Fm) / da, (Fp - F0) / db
                v = (da * sb + db * sa) / (da + db)
                lim = 3.0 * np.minimum(np.abs(sa), np.abs(sb))
                v = np.where(v > lim, lim, np.where(v < -lim, -lim, v))
            v = np.where(np.isnan(Fm) | np.isnan(Fp) | np.isnan(F0), 0.0, v)
            idx = [slice(None)] * F.ndim
            idx[F.ndim - 1 - d] = slice(1, n - 1)
            D[tuple(idx)] = v
        diffs.append(D)
    return diffs


def smooth_spline_diffs(axes, F):
    """Node derivatives along every axis for the "smooth_spline" interpolation
    (spline::computeDiffs, plask/mesh/rectangular_spline.cpp:440-600), without symmetry or
    periodicity: the cubic spline with continuous second derivatives and zero slopes at the
    first and last node, db s[i-1] + 2 (da + db) s[i] + da s[i+1] =
    3 (da/db (y[i+1] - y[i]) + db/da (y[i] - y[i-1])), solved per mesh line."""
    from scipy.linalg import solve_banded

    diffs = []
    for d, a in enumerate(axes):
        n = a.size
        if n < 3:
            diffs.append(np.zeros_like(F))
            continue
        nd = F.ndim - 1 - d
        Y = np.moveaxis(F, nd, 0).reshape(n, -1)
        h = np.diff(a)
        da, db = h[:-1], h[1:]
        ab = np.zeros((3, n))
        ab[1, 0] = ab[1, -1] = 1.0
        ab[0, 2:] = da            # super-diagonal: du[i] = da of row i
        ab[1, 1:-1] = 2.0 * (da + db)
        ab[2, :-2] = db           # sub-diagonal: dl[i-1] = db of row i
        rhs = np.zeros_like(Y)
        rhs[1:-1] = 3.0 * ((da / db)[:, None] * (Y[2:] - Y[1:-1]) + (db / da)[:, None] * (Y[1:-1] - Y[:-2]))
        S = solve_banded((1, 1), ab, rhs)
        diffs.append(np.moveaxis(S.reshape((n,) + np.moveaxis(F, nd, 0).shape[1:]), 0, nd))
    return diffs


def _hermite(x, dlen):
    """Cubic Hermite basis (values at the low and high node, slopes times the interval)."""
    return (((2.0 * x - 3.0) * x * x + 1.0), ((-2.0 * x + 3.0) * x * x),
            (((x - 2.0) * x + 1.0) * x * dlen), ((x - 1.0) * x * x * dlen))


def _spline_combine(F, diffs, lo, hi, x, dlen):
    """The spline formula of SplineRect2D/3DLazyDataImpl::at (rectangular_spline.cpp:30-237):
    products of the value bases at the element's corners, plus along each axis the slope
    bases times the corner derivatives weighted by the value bases of the other axes."""
    dims = len(lo)
    H = [_hermite(x[d], dlen[d]) for d in range(dims)]
    val = 0.0
    for c in itertools.product((0, 1), repeat=dims):
        w = 1.0
        for d in range(dims):
            w = w * H[d][c[d]]
        val = val + w * F[tuple((hi[d] if c[d] else lo[d]) for d in range(dims))[::-1]]
    for d in range(dims):
        others = [e for e in range(dims) if e != d]
        for c in itertools.product((0, 1), repeat=dims - 1):
            w = 1.0
            for e, ce in zip(others, c):
                w = w * H[e][ce]
            at = {e: (hi[e] if ce else lo[e]) for e, ce in zip(others, c)}
            il = tuple((lo[k] if k == d else at[k]) for k in range(dims))[::-1]
            ih = tuple((hi[k] if k == d else at[k]) for k in range(dims))[::-1]
            val = val + w * (H[d][2] * diffs[d][il] + H[d][3] * diffs[d][ih])
    return val


def spline_interpolate(axes, F, pts, method, active=None):
    """Spline interpolation of nodal values on a rectilinear mesh ("spline": Hyman-filtered
    parabolic slopes; "smooth_spline": the C2 spline, full meshes only).  A full mesh
    brackets each coordinate as prepareInterpolationForAxis does (plask/mesh/axis1d.cpp:
    99-154: outside the axis both nodes are the edge node, 1 um apart); a masked mesh
    (``active``) uses the holding element of its element search and gives NaN where there
    is none."""
    dims = len(axes)
    if active is not None and method != "spline":
        raise BadInput(-1, f"{method} interpolation is not provided on masked meshes (the reference has the Hyman spline only)")
    diffs = hyman_diffs(axes, F) if method == "spline" else smooth_spline_diffs(axes, F)
    out = np.full(len(pts), np.nan)
    if active is None:
        sel = np.arange(len(pts))
        lo, hi, lo_c, hi_c = [], [], [], []
        for d, a in enumerate(axes):
            xd = pts[:, d]
            n = a.size
            up = np.searchsorted(a, xd, side="right")
            lo.append(np.where(up == 0, 0, up - 1))
            lo_c.append(np.where(up == 0, a[0] - 1.0, a[np.maximum(up - 1, 0)]))
            hi.append(np.where(up == n, n - 1, up))
            hi_c.append(np.where(up == n, a[n - 1] + 1.0, a[np.minimum(up, n - 1)]))
    else:
        elem, found = masked_element_search(axes, active, pts)
        sel = np.flatnonzero(found)
        lo = [elem[d][sel] for d in range(dims)]
        hi = [lo[d] + 1 for d in range(dims)]
        lo_c = [axes[d][lo[d]] for d in range(dims)]
        hi_c = [axes[d][hi[d]] for d in range(dims)]
    dlen = [hi_c[d] - lo_c[d] for d in range(dims)]
    x = [(pts[sel, d] - lo_c[d]) / dlen[d] for d in range(dims)]
    out[sel] = _spline_combine(F, diffs, lo, hi, x, dlen)
    return out


def _element_axis(axis, x):
    """Index of the element holding x, clamped to the mesh (findUpIndex - 1)."""
    return np.clip(np.searchsorted(axis, x, side="right") - 1, 0, axis.size - 2)


_METHODS = {"default": "linear", None: "linear", "linear": "linear", "nearest": "nearest", "spline": "spline",
            "smooth_spline": "smooth_spline", "smooth spline": "smooth_spline"}


def _check_interpolation(method, splines=False):
    """PLaSK's interpolation method names (plask/mesh/interpolation.cpp:18-28, lower case);
    ``splines``: the provider also offers "spline" (Hyman-filtered) and "smooth_spline"."""
    key = method.lower() if isinstance(method, str) else method
    m = _METHODS.get(key)
    if m is None or (not splines and m in ("spline", "smooth_spline")):
        names = "linear, nearest, spline or smooth_spline" if splines else "linear or nearest"
        raise BadInput(-1, f"unsupported interpolation {method!r} ({names})")
    return m


def _interp_axis(axis, x):
    """Bracketing indices and weights of points x on an increasing axis (clamped)."""
    i = np.clip(np.searchsorted(axis, x, side="right") - 1, 0, axis.size - 2)
    w = (x - axis[i]) / (axis[i + 1] - axis[i])
    inside = (x >= axis[0]) & (x <= axis[-1])
    return i, np.clip(w, 0.0, 1.0), inside


def save_state(solver, path):
    """Write the solver's temperature field (masked-mesh numbering, mesh order) with the
    mesh axes and iteration order to the ``.npz`` file ``path``: a checkpoint for
    :func:`load_state`.  The reference keeps the temperatures between ``compute()`` calls
    until ``invalidate()`` (therm3d.cpp:118-122); this makes that warm restart survive the
    process."""
    solver.initialize()
    data = {"temperature": solver._fem.temperature(), "ordering": np.array(solver.mesh.ordering),
            "solver": np.array(type(solver).__name__)}
    for d, a in enumerate(solver.mesh.axes):
        data[f"axis{d}"] = np.asarray(a, np.float64)
    np.savez(path, **data)


def load_state(solver, path):
    """Restore a temperature field written by :func:`save_state` as the starting field of
    the next ``compute()``.  The mesh (axes and iteration order) must be the one saved;
    the field must have the solver's node count (the same masked mesh)."""
    with np.load(path) as f:
        axes = [f[k] for k in sorted(k for k in f.files if k.startswith("axis"))]
        ordering = str(f["ordering"])
        T = np.array(f["temperature"], np.float64)
    mine = [np.asarray(a, np.float64) for a in solver.mesh.axes]
    if len(axes) != len(mine) or any(a.shape != b.shape or not np.array_equal(a, b) for a, b in zip(axes, mine)):
        raise BadInput(-1, f"{solver.id}: the saved field belongs to another mesh")
    if ordering != solver.mesh.ordering:
        raise BadInput(-1, f"{solver.id}: the saved field has iteration order {ordering}, "
                           f"the mesh {solver.mesh.ordering}")
    solver.initialize()
    nn, _ = solver._fem.sizes()
    if T.size != nn:
        raise BadInput(-1, f"{solver.id}: the saved field has {T.size} nodes, the masked mesh {nn}")
    solver._fem.set_temperature(T)


class Static3D:
    """Finite element thermal solver for 3D geometry, computed on the GPU.

    Attributes (therm_python.cpp:136-151, fem/python.hpp:31-41, therm3d.cpp:20-33):
    ``geometry``, ``mesh``, ``inittemp`` (300 K), ``maxerr`` (0.05 K),
    ``algorithm`` ("iterative"; also "cholesky", "gauss", "gpu-pcg",
    "gpu-mixed", "gpu-learned"), ``iterative`` (maxit, maxerr, noconv, ...),
    ``empty_elements`` ("default", "exclude", "include"), the four
    boundary-condition lists, ``inHeat``/``inHeatDensity`` and the providers
    ``outTemperature``, ``outHeatFlux``, ``outThermalConductivity``.

    Extra GPU knobs: ``rtol`` (FP64 relative residual of every linear solve,
    default 1e-14), ``residual_norm`` ("plain": 2-norm, the default; "scaled":
    Jacobi-weighted, for strong conductivity contrast) and ``bc_compat`` (True: the reference's placement of 3D
    face boundary terms).
    """

    def __init__(self, name=""):
        self.name = name
        self._geometry = None
        self._mesh = None
        self.inittemp = 300.0
        self.maxerr = 0.05
        self._algorithm = "iterative"
        self.iterative = IterativeParams()
        self._empty_elements = "default"
        self.rtol = 1e-14
        self.residual_norm = "plain"
        self.bc_compat = True
        self.temperature_boundary = BoundaryConditions(self, _native.BC_TEMPERATURE, 1)
        self.heatflux_boundary = BoundaryConditions(self, _native.BC_HEATFLUX, 1)
        self.convection_boundary = BoundaryConditions(self, _native.BC_CONVECTION, 2)
        self.radiation_boundary = BoundaryConditions(self, _native.BC_RADIATION, 2)
        self._inHeat = Receiver(self)
        self.outTemperature = Provider(self._get_temperatures)
        self.outHeatFlux = Provider(self._get_heat_fluxes)
        self.outThermalConductivity = Provider(self._get_conductivity)
        self._fem = None
        self._elements_dirty = True
        self._bc_dirty = True
        self._heat_dirty = True
        self._toterr = 0.0
        self.stats = {}
        self.loop_log = []
        self._preconditioner = None

    # ---------------------------------------------------------------- properties
    @property
    def id(self):
        return f"{self.name}:thermal.Static3D" if self.name else "thermal.Static3D"

    @property
    def geometry(self):
        return self._geometry

    @geometry.setter
    def geometry(self, g):
        self._geometry = g
        self.invalidate()
        self._elements_dirty = True

    @property
    def mesh(self):
        return self._mesh

    @mesh.setter
    def mesh(self, m):
        self._mesh = m
        self.invalidate()
        self._fem = None

    @property
    def algorithm(self):
        return self._algorithm

    @algorithm.setter
    def algorithm(self, a):
        if a not in _native.ALGORITHMS:
            raise BadInput(-1, f"unknown algorithm {a!r}")
        self._algorithm = a

    @property
    def empty_elements(self):
        return self._empty_elements

    @empty_elements.setter
    def empty_elements(self, v):
        if v not in _native.EMPTY:
            raise BadInput(-1, f"unknown empty_elements {v!r}")
        self._empty_elements = v
        self.invalidate()

    @property
    def preconditioner(self):
        """Learned preconditioner (plask_gb300._native.UNet) used by algorithm "gpu-learned"."""
        return self._preconditioner

    @preconditioner.setter
    def preconditioner(self, net):
        self._preconditioner = net
        if self._fem is not None:
            _native.attach_preconditioner(self._fem, net)

    @property
    def inHeat(self):
        return self._inHeat

    @inHeat.setter
    def inHeat(self, v):
        self._inHeat.attach(v)

    inHeatDensity = inHeat

    @property
    def err(self):
        """Maximum estimated error of the last compute() (therm3d.hpp:111)."""
        return self._toterr

    # ---------------------------------------------------------------- lifecycle
    def _bc_changed(self):
        self._bc_dirty = True

    def _heat_changed(self):
        self._heat_dirty = True

    def initialize(self):
        if self._geometry is None:
            raise BadInput(-1, f"{self.id}: No geometry specified")
        if self._mesh is None:
            raise BadInput(-1, f"{self.id}: No mesh specified")
        if self._fem is None:
            self._fem = _native.Fem3D(self._mesh.axes, self._mesh.ordering)
            self._fem.set_log_callback(self._log)
            self._elements_dirty = self._bc_dirty = self._heat_dirty = True
            if self._preconditioner is not None:
                _native.attach_preconditioner(self._fem, self._preconditioner)
        fem = self._fem
        if self._elements_dirty:
            mt = self._geometry.materials
            fem.set_materials(mt.k300, mt.p, mt.kz_ratio, mt.hexp, mt.empty)
            mt.apply_tables(fem)
            mat = self._geometry.material_ids(self._mesh)
            leaf = self._geometry.leaf_height(self._mesh)
            order = self._mesh.ordering
            fem.set_elements(to_mesh_order(mat, order), to_mesh_order(self._inHeat(self._mesh), order),
                             None if leaf is None else to_mesh_order(leaf, order))
            self._elements_dirty = False
            self._heat_dirty = False
        elif self._heat_dirty:
            fem.set_heat(to_mesh_order(self._inHeat(self._mesh), self._mesh.ordering))
            self._heat_dirty = False
        if self._bc_dirty:
            for kind, lst in ((_native.BC_TEMPERATURE, self.temperature_boundary),
                              (_native.BC_HEATFLUX, self.heatflux_boundary),
                              (_native.BC_CONVECTION, self.convection_boundary),
                              (_native.BC_RADIATION, self.radiation_boundary)):
                fem.clear_bc(kind)
                for place, vals in lst:
                    nodes = place.nodes(self._mesh) if hasattr(place, "nodes") else np.asarray(place, np.int64)
                    fem.add_bc(kind, nodes, *vals)
            self._bc_dirty = False
        it = self.iterative
        maxit = it.maxit if self._algorithm == "iterative" and it.maxit != 1000 else 0
        fem.set_solver(self._algorithm, self.rtol, maxit, it.noconv, self._empty_elements, self.bc_compat)
        fem.set_residual_norm(self.residual_norm)
        fem.set_loop(self.inittemp, self.maxerr)

    def invalidate(self):
        """Forget the computed temperatures (therm3d.cpp:118-122)."""
        if self._fem is not None:
            self._fem.invalidate()
        self._elements_dirty = True

    def _log(self, level, msg):
        if msg.startswith("Loop "):
            self.loop_log.append(msg)
        lvl = {2: logging.WARNING, 3: logging.INFO, 4: logging.INFO}.get(level, logging.DEBUG)
        log.log(lvl, "%s: %s", self.id, msg)

    # ---------------------------------------------------------------- computation
    def compute(self, loops=0):
        """Run thermal calculations; returns the maximum temperature correction (therm3d.cpp:281-340)."""
        self.initialize()
        self.loop_log = []
        tot, st = self._fem.compute(loops)
        self._toterr = tot
        self.stats = st
        self.iterative.converged = bool(st["converged"])
        self.iterative.iters = st["inner_iterations"]
        self.iterative.err = st["last_rel_residual"]
        return tot

    # ---------------------------------------------------------------- results
    def temperatures(self):
        """Nodal temperatures in the solver's numbering (masked mesh, mesh order)."""
        self.initialize()
        return self._fem.temperature()

    def save(self, path):
        """Checkpoint the temperature field to an ``.npz`` file (:func:`save_state`)."""
        save_state(self, path)

    def load(self, path):
        """Start the next ``compute()`` from a checkpointed field (:func:`load_state`)."""
        load_state(self, path)

    def _full_temperature(self):
        """Canonical (n2, n1, n0) temperature with NaN at nodes outside the masked mesh."""
        t = self._fem.temperature()
        n = len(self._mesh)
        canon_idx = self._mesh.index_array().ravel()
        full = np.full(n, np.nan)
        if t.size == n:
            full = t[canon_idx]
        else:
            nn, _ = self._fem.sizes()
            # masked numbering: active nodes in mesh order
            act = self._active_mask_mesh_order()
            vals = np.full(n, np.nan)
            vals[np.flatnonzero(act)] = t
            full = vals[canon_idx]
        return full.reshape(self._mesh.shape)

    def _active_elements(self):
        """Canonical mask of the masked mesh's elements (fem_solver.hpp:164-189: empty
        elements are left out unless included, by default with the iterative algorithm)."""
        mat = self._geometry.material_ids(self._mesh)
        mt = self._geometry.materials
        excl = self._empty_elements in ("exclude", "excluded") or (
            self._empty_elements == "default" and self._algorithm != "iterative")
        return ~mt.empty[mat] if excl else np.ones(mat.shape, bool)

    def _active_mask_mesh_order(self):
        mesh = self._mesh
        act_el = self._active_elements()
        n2, n1, n0 = mesh.shape
        used = np.zeros(mesh.shape, bool)
        for ck in (0, 1):
            for cj in (0, 1):
                for ci in (0, 1):
                    used[ck:n2 - 1 + ck, cj:n1 - 1 + cj, ci:n0 - 1 + ci] |= act_el
        return to_mesh_order(used, mesh.ordering)

    def _wrap(self, pts):
        """Points as the providers see them (InterpolationFlags::wrap,
        plask/mesh/interpolation.hpp:232-250): along an axis the geometry mirrors at 0 a
        negative coordinate reads at its absolute value.  Returns the wrapped points and, per
        mirrored axis, the mask of reflected points."""
        sym = tuple(getattr(self._geometry, "symmetric", ())) if self._geometry is not None else ()
        if not any(sym):
            return pts, {}
        return wrap_symmetric(pts, sym, [float(a[0]) for a in self._mesh.axes], [float(a[-1]) for a in self._mesh.axes])

    def _get_temperatures(self, dst_mesh, interpolation="linear"):
        """Temperatures on a destination mesh (therm3d.cpp:387-395): trilinear or the nearest
        node, the edge values continuing outside the mesh; on a masked mesh its element
        search, 300 K where no included element holds the point."""
        if self._fem is None:
            n = len(dst_mesh) if dst_mesh is not None else 0
            return np.full(n, self.inittemp)
        T = self._full_temperature()
        if dst_mesh is None:
            return T
        pts, _ = self._wrap(_points(dst_mesh))
        method = _check_interpolation(interpolation, splines=True)
        active = self._active_elements()
        masked = not np.all(active)
        if method in ("spline", "smooth_spline"):
            out = spline_interpolate(self._mesh.axes, T, pts, method, active if masked else None)
            return np.where(np.isnan(out), 300.0, out)
        if masked:
            # the masked mesh's interpolation; NaN (no included element) reads 300 K (SafeData)
            out = masked_interpolate(self._mesh.axes, T, active, pts, method)
            return np.where(np.isnan(out), 300.0, out)
        if method == "nearest":
            # the nearest node (rectilinear3d.hpp:853-860)
            i0, i1, i2 = (_nearest_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            out = T[i2, i1, i0]
            return np.where(np.isnan(out), 300.0, out)
        return _trilinear(self._mesh.axes, T, pts, fill=None)

    def heat_fluxes(self):
        """Per-element heat flux [W/m^2], canonical (ne2, ne1, ne0, 3) (saveHeatFluxes)."""
        self.initialize()
        q = self._fem.heat_flux()
        eidx = self._mesh.element_index_array().ravel()
        return q[eidx].reshape(self._mesh.element_shape + (3,))

    def _get_heat_fluxes(self, dst_mesh, interpolation="linear"):
        """Heat flux on a destination mesh (therm3d.cpp:398-411): linear over the element
        midpoints or the holding element, the edge values continuing outside; on a masked
        mesh its element mesh's interpolation, 0 where no included element holds the point."""
        if self._fem is None:
            n = len(dst_mesh) if dst_mesh is not None else 0
            return np.zeros((n, 3))
        q = np.nan_to_num(self.heat_fluxes())
        if dst_mesh is None:
            return q
        mids = [0.5 * (a[1:] + a[:-1]) for a in self._mesh.axes]
        pts, flips = self._wrap(_points(dst_mesh))
        active = self._active_elements()
        method = _check_interpolation(interpolation, splines=True)
        if method in ("spline", "smooth_spline"):
            if not np.all(active):
                raise BadInput(-1, f"{self.id}: spline interpolation of heat fluxes on a masked mesh is not provided")
            out = np.stack([spline_interpolate(mids, q[..., c], pts, method) for c in range(3)], axis=-1)
        elif not np.all(active):
            # the masked element mesh's interpolation; NaN reads 0 (SafeData)
            out = np.nan_to_num(masked_element_interpolate(self._mesh.axes, q, active, pts, method))
        elif method == "nearest":
            # the element holding the point (the reference's element-mesh lookup,
            # rectilinear3d.hpp:282-297, searches axis 0 for the second coordinate as well;
            # that slip is not reproduced)
            i0, i1, i2 = (_element_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            out = q[i2, i1, i0].copy()
        else:
            out = np.stack([_trilinear(mids, q[..., c], pts, fill=None) for c in range(3)], axis=-1)
        for d, m in flips.items():  # the normal component of a mirrored point (Symmetry NPP / PNP / PPN)
            out[m, d] *= -1.0
        return out

    def _get_conductivity(self, dst_mesh, interpolation="linear"):
        """(k_xy, k_z) of the element holding each point (therm3d.cpp:421-435)."""
        self.initialize()
        k = self._fem.conductivity()
        eidx = self._mesh.element_index_array().ravel()
        k = k[eidx].reshape(self._mesh.element_shape + (2,))
        if dst_mesh is None:
            return k
        idx, ok = conductivity_elements(self._mesh.axes, self._wrap(_points(dst_mesh))[0])
        out = k[idx[2], idx[1], idx[0]]
        out[~ok] = np.nan
        return out

    def thickness(self):
        """Layer-run thickness per element, canonical shape (onInitialize, therm3d.cpp:81-113)."""
        self.initialize()
        th = self._fem.thickness()
        eidx = self._mesh.element_index_array().ravel()
        return th[eidx].reshape(self._mesh.element_shape)


class Dynamic3D(Static3D):
    """Finite element time-stepping thermal solver for 3D geometry, on the GPU.

    A drop-in for PLaSK's ``thermal.dynamic.Dynamic3D`` (femT3d.cpp,
    python/dynamic_python.cpp:70-90): ``compute(time)`` advances ``time`` ns with the theta
    method; attributes ``inittemp`` (300 K), ``timestep`` (0.1 ns), ``methodparam``
    (0.5: Crank-Nicolson), ``lumping`` (True: lumped heat capacity; False: the consistent
    matrix), ``rebuildfreq`` (0), ``logfreq`` (500), ``time`` / ``elapsed_time`` (read only,
    python/dynamic_python.cpp:86-87),
    ``algorithm`` ("iterative"), ``temperature_boundary``, ``inHeat`` and the providers
    of Static3D.  The material table must carry ``cp`` and ``dens``.
    """

    def __init__(self, name=""):
        super().__init__(name)
        self.timestep = 0.1
        self.methodparam = 0.5
        self.lumping = True
        self.rebuildfreq = 0
        self.logfreq = 500
        self._elapstime = 0.0
        # the time-stepping solver has temperature conditions only (femT3d.hpp:54)
        del self.heatflux_boundary, self.convection_boundary, self.radiation_boundary
        self.heatflux_boundary = self.convection_boundary = self.radiation_boundary = ()

    @property
    def id(self):
        return f"{self.name}:thermal.Dynamic3D" if self.name else "thermal.Dynamic3D"

    @property
    def time(self):
        """Time of calculations performed so far since the last invalidation [ns]."""
        return self._elapstime

    elapsed_time = time

    def compute(self, time):
        """Run thermal calculations for ``time`` ns (femT3d.cpp:255-315)."""
        self.initialize()
        mt = self._geometry.materials
        if mt.cp is None or mt.dens is None:
            raise BadInput(-1, f"{self.id}: the material table has no cp / dens")
        self._fem.set_dynamic(mt.cp, mt.dens, self.timestep, self.methodparam, self.lumping, self.rebuildfreq,
                              self.logfreq)
        self.loop_log = []
        el, st = self._fem.compute_dynamic(time)
        self._elapstime = el
        self.stats = st
        self.iterative.converged = bool(st["converged"])
        self.iterative.iters = st["inner_iterations"]
        return 0.0


def _points(dst):
    if isinstance(dst, RectangularMesh3D):
        Z, Y, X = np.meshgrid(dst.axis2, dst.axis1, dst.axis0, indexing="ij")
        pts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
        order = dst.index_array().ravel()
        out = np.empty_like(pts)
        out[order] = pts
        return out
    return np.asarray(dst, np.float64).reshape(-1, 3)


def _trilinear(axes, F, pts, fill, clamp=False, box=None):
    """Trilinear interpolation of canonical F (n2, n1, n0) at points (m, 3).  Outside the
    axes the edge values continue (prepareInterpolationForAxis, plask/mesh/axis1d.cpp:99-154,
    gives both bracketing nodes the edge index); ``fill`` (unless None) replaces the values
    of points outside the axes (or outside ``box`` with ``clamp``)."""
    ii, ww, ok = [], [], np.ones(len(pts), bool)
    for d in range(3):
        a = axes[d]
        if a.size == 1:
            i = np.zeros(len(pts), np.int64)
            w = np.zeros(len(pts))
            inside = np.ones(len(pts), bool)
        else:
            i, w, inside = _interp_axis(a, pts[:, d])
        if clamp:
            b = box[d]
            inside = (pts[:, d] >= b[0]) & (pts[:, d] <= b[-1])
        ii.append(i)
        ww.append(w)
        ok &= inside
    out = np.zeros(len(pts))
    for ck in (0, 1):
        for cj in (0, 1):
            for ci in (0, 1):
                wt = (ww[0] if ci else 1 - ww[0]) * (ww[1] if cj else 1 - ww[1]) * (ww[2] if ck else 1 - ww[2])
                k = np.minimum(ii[2] + ck, F.shape[0] - 1)
                j = np.minimum(ii[1] + cj, F.shape[1] - 1)
                i = np.minimum(ii[0] + ci, F.shape[2] - 1)
                out += wt * F[k, j, i]
    if fill is not None:
        out[~ok] = fill
    return out


def solver_for_structure(s, ordering="best", algorithm="gpu-mixed", name="", **kw):
    """A configured :class:`Static3D` for a generated structure (plask_gb300.structures)."""
    mesh = RectangularMesh3D(*s.axes, ordering=ordering)
    sv = Static3D(name)
    sv.geometry = StructureGeometry.from_structure(s)
    sv.mesh = mesh
    sv.inHeat = s.heat
    sv.inittemp = s.inittemp
    sv.maxerr = s.maxerr
    sv.algorithm = algorithm
    for side, v in s.temperature:
        sv.temperature_boundary.append(RectangularMesh3D.side(side), v)
    for side, v in s.heatflux:
        sv.heatflux_boundary.append(RectangularMesh3D.side(side), v)
    for side, h, ta in s.convection:
        sv.convection_boundary.append(RectangularMesh3D.side(side), {"coeff": h, "ambient": ta})
    for side, e, ta in s.radiation:
        sv.radiation_boundary.append(RectangularMesh3D.side(side), {"emissivity": e, "ambient": ta})
    for k, v in kw.items():
        setattr(sv, k, v)
    return sv
