"""Rectilinear 3D and 2D meshes with PLaSK's iteration orders and named boundaries.

Mirrors the parts of ``plask.mesh.Rectangular3D`` that the Static3D path uses
(plask/mesh/rectilinear3d.hpp, rectilinear3d.cpp:20-190):

* node index in iteration order ``ORDER_<major><medium><minor>``:
  ``i_minor + n_minor * (i_medium + n_medium * i_major)``;
* elements numbered the same way over ``n - 1`` cells per axis;
* boundaries Back/Front (axis 0 lo/hi), Left/Right (axis 1 lo/hi),
  Bottom/Top (axis 2 lo/hi), their unions, and index boxes;
* ``setOptimalIterationOrder`` (largest axis major, smallest minor).

Arrays called "canonical" here have shape (n2, n1, n0) -- axis 0 fastest --
which is also the device layout of the GPU solver.  The 2D mesh
(``RectangularMesh2D``, plask/mesh/rectangular2d.hpp/.cpp) has orders ORDER_10
(axis 0 fastest) and ORDER_01 (axis 1 fastest) and canonical shape (n1, n0).
"""
from __future__ import annotations

import numpy as np

ORDERS = ("012", "021", "102", "120", "201", "210")


def optimal_order(n0, n1, n2):
    """Iteration order with the longest axis major (rectilinear3d.cpp:74-85)."""
    n = (n0, n1, n2)
    for f, s, t in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        if n[t] <= n[s] <= n[f]:
            return f"{f}{s}{t}"
    return "210"


def order_strides(sizes, order):
    """Strides (s0, s1, s2) of axes 0/1/2 in a mesh-order array of extents ``sizes``."""
    a, b, c = (int(ch) for ch in order)
    s = [0, 0, 0]
    s[c] = 1
    s[b] = sizes[c]
    s[a] = sizes[c] * sizes[b]
    return tuple(s)


def mesh_index(sizes, order):
    """Canonical-shaped (n2, n1, n0) array holding each point's mesh-order index."""
    s0, s1, s2 = order_strides(sizes, order)
    n0, n1, n2 = sizes
    return (np.arange(n2)[:, None, None] * s2 + np.arange(n1)[None, :, None] * s1
            + np.arange(n0)[None, None, :] * s0).astype(np.int64)


def to_mesh_order(canon, order, comps=None):
    """Flatten a canonical (n2, n1, n0[, c]) array into mesh order."""
    canon = np.asarray(canon)
    shp = canon.shape[:3]
    sizes = (shp[2], shp[1], shp[0])
    idx = mesh_index(sizes, order).ravel()
    tail = canon.shape[3:]
    out = np.empty((idx.size,) + tail, dtype=canon.dtype)
    out[idx] = canon.reshape((idx.size,) + tail)
    return out


def from_mesh_order(flat, sizes, order):
    """Inverse of :func:`to_mesh_order` for extents ``sizes`` = (n0, n1, n2)."""
    flat = np.asarray(flat)
    idx = mesh_index(sizes, order).ravel()
    tail = flat.shape[1:]
    return flat[idx].reshape((sizes[2], sizes[1], sizes[0]) + tail)


class Boundary:
    """A set of mesh nodes, resolved lazily against a mesh (boundary.hpp)."""

    def __init__(self, fn, name=""):
        self._fn = fn
        self.name = name

    def mask(self, mesh):
        """Boolean canonical node mask."""
        return self._fn(mesh)

    def nodes(self, mesh):
        """Mesh-order indices of the nodes, ascending."""
        m = self.mask(mesh)
        return np.sort(mesh.index_array()[m])

    def __or__(self, other):
        return Boundary(lambda mesh: self.mask(mesh) | other.mask(mesh), f"{self.name}|{other.name}")

    __add__ = __or__

    def __and__(self, other):
        return Boundary(lambda mesh: self.mask(mesh) & other.mask(mesh), f"{self.name}&{other.name}")

    def __sub__(self, other):
        return Boundary(lambda mesh: self.mask(mesh) & ~other.mask(mesh), f"{self.name}-{other.name}")

    def __repr__(self):
        return f"<Boundary {self.name}>"


def _side(sl, name):
    def fn(mesh):
        m = np.zeros(mesh.shape, bool)
        m[sl] = True
        return m

    return Boundary(fn, name)


class RectangularMesh3D:
    """Rectilinear 3D mesh: three increasing axes in micrometres and an iteration order."""

    def __init__(self, axis0, axis1, axis2, ordering=None):
        self.axis0 = np.ascontiguousarray(axis0, dtype=np.float64)
        self.axis1 = np.ascontiguousarray(axis1, dtype=np.float64)
        self.axis2 = np.ascontiguousarray(axis2, dtype=np.float64)
        for a in self.axes:
            if a.ndim != 1 or a.size < 2 or np.any(np.diff(a) <= 0):
                raise ValueError("mesh axes must be strictly increasing with at least 2 points")
        if ordering is None:
            ordering = "012"
        if ordering == "best":
            ordering = optimal_order(*self.sizes)
        if ordering not in ORDERS:
            raise ValueError(f"unknown iteration order {ordering!r}")
        self.ordering = ordering

    @property
    def axes(self):
        return (self.axis0, self.axis1, self.axis2)

    @property
    def sizes(self):
        return tuple(a.size for a in self.axes)

    @property
    def shape(self):
        """Canonical node shape (n2, n1, n0)."""
        n0, n1, n2 = self.sizes
        return (n2, n1, n0)

    @property
    def element_shape(self):
        n2, n1, n0 = self.shape
        return (n2 - 1, n1 - 1, n0 - 1)

    def __len__(self):
        return int(np.prod(self.sizes))

    @property
    def elements_count(self):
        return int(np.prod([n - 1 for n in self.sizes]))

    def set_optimal_ordering(self):
        self.ordering = optimal_order(*self.sizes)

    def index_array(self):
        return mesh_index(self.sizes, self.ordering)

    def element_index_array(self):
        return mesh_index(tuple(n - 1 for n in self.sizes), self.ordering)

    def element_midpoints(self):
        """Canonical (ne2, ne1, ne0, 3) array of element midpoints."""
        m = [0.5 * (a[1:] + a[:-1]) for a in self.axes]
        Z, Y, X = np.meshgrid(m[2], m[1], m[0], indexing="ij")
        return np.stack([X, Y, Z], axis=-1)

    # named boundaries (rectilinear3d.cpp:158-190)
    @staticmethod
    def Back():
        return _side((slice(None), slice(None), 0), "back")

    @staticmethod
    def Front():
        return _side((slice(None), slice(None), -1), "front")

    @staticmethod
    def Left():
        return _side((slice(None), 0), "left")

    @staticmethod
    def Right():
        return _side((slice(None), -1), "right")

    @staticmethod
    def Bottom():
        return _side((0,), "bottom")

    @staticmethod
    def Top():
        return _side((-1,), "top")

    @staticmethod
    def IndexBox(i0, i1, j0, j1, k0, k1):
        """Nodes with index ranges [i0, i1] x [j0, j1] x [k0, k1] (inclusive)."""
        return _side((slice(k0, k1 + 1), slice(j0, j1 + 1), slice(i0, i1 + 1)), "box")

    @staticmethod
    def Nodes(mask):
        """Explicit canonical node mask."""
        mask = np.asarray(mask, bool)
        return Boundary(lambda mesh: mask.reshape(mesh.shape), "nodes")

    @staticmethod
    def side(name):
        return {"back": RectangularMesh3D.Back, "front": RectangularMesh3D.Front, "left": RectangularMesh3D.Left,
                "right": RectangularMesh3D.Right, "bottom": RectangularMesh3D.Bottom,
                "top": RectangularMesh3D.Top}[name]()


# ----------------------------------------------------------------------------------------
# 2D


ORDERS2D = ("10", "01")


def optimal_order2d(n0, n1):
    """RectangularMesh2D::setOptimalIterationOrder (rectangular2d.hpp:296-298): the longer axis major."""
    return "01" if n0 > n1 else "10"


def mesh_index2d(sizes, order):
    """Canonical-shaped (n1, n0) array of mesh-order indices (rectangular2d.cpp:20-38):
    ORDER_10 index = i0 + n0 i1, ORDER_01 index = i1 + n1 i0."""
    n0, n1 = sizes
    i0 = np.arange(n0)[None, :]
    i1 = np.arange(n1)[:, None]
    if order == "10":
        return (i0 + n0 * i1).astype(np.int64)
    if order == "01":
        return (i1 + n1 * i0).astype(np.int64)
    raise ValueError(f"unknown 2D iteration order {order!r}")


def to_mesh_order2d(canon, order, comps=None):
    """Flatten a canonical (n1, n0[, c]) array into mesh order."""
    canon = np.asarray(canon)
    sizes = (canon.shape[1], canon.shape[0])
    idx = mesh_index2d(sizes, order).ravel()
    tail = canon.shape[2:]
    out = np.empty((idx.size,) + tail, dtype=canon.dtype)
    out[idx] = canon.reshape((idx.size,) + tail)
    return out


class RectangularMesh2D:
    """Rectilinear 2D mesh (plask.mesh.Rectangular2D): axis 0 horizontal (the radius of a
    cylindrical geometry), axis 1 vertical, micrometres, with an iteration order
    "01" (default, axis 1 fastest), "10" or "best"."""

    def __init__(self, axis0, axis1, ordering=None):
        self.axis0 = np.ascontiguousarray(axis0, dtype=np.float64)
        self.axis1 = np.ascontiguousarray(axis1, dtype=np.float64)
        for a in self.axes:
            if a.ndim != 1 or a.size < 2 or np.any(np.diff(a) <= 0):
                raise ValueError("mesh axes must be strictly increasing with at least 2 points")
        if ordering is None:
            ordering = "01"
        if ordering == "best":
            ordering = optimal_order2d(*self.sizes)
        if ordering not in ORDERS2D:
            raise ValueError(f"unknown iteration order {ordering!r}")
        self.ordering = ordering

    @property
    def axes(self):
        return (self.axis0, self.axis1)

    @property
    def sizes(self):
        return (self.axis0.size, self.axis1.size)

    @property
    def shape(self):
        """Canonical node shape (n1, n0)."""
        return (self.axis1.size, self.axis0.size)

    @property
    def element_shape(self):
        return (self.axis1.size - 1, self.axis0.size - 1)

    def __len__(self):
        return self.axis0.size * self.axis1.size

    @property
    def elements_count(self):
        return (self.axis0.size - 1) * (self.axis1.size - 1)

    def index_array(self):
        return mesh_index2d(self.sizes, self.ordering)

    def element_index_array(self):
        return mesh_index2d((self.axis0.size - 1, self.axis1.size - 1), self.ordering)

    def element_midpoints(self):
        """Canonical (ne1, ne0, 2) array of element midpoints."""
        m0 = 0.5 * (self.axis0[1:] + self.axis0[:-1])
        m1 = 0.5 * (self.axis1[1:] + self.axis1[:-1])
        Y, X = np.meshgrid(m1, m0, indexing="ij")
        return np.stack([X, Y], axis=-1)

    # named boundaries (rectangular2d.hpp: left/right along axis 0, bottom/top along axis 1)
    @staticmethod
    def Left():
        return _side((slice(None), 0), "left")

    @staticmethod
    def Right():
        return _side((slice(None), -1), "right")

    @staticmethod
    def Bottom():
        return _side((0,), "bottom")

    @staticmethod
    def Top():
        return _side((-1,), "top")

    @staticmethod
    def IndexBox(i0, i1, j0, j1):
        """Nodes with index ranges [i0, i1] x [j0, j1] (inclusive)."""
        return _side((slice(j0, j1 + 1), slice(i0, i1 + 1)), "box")

    @staticmethod
    def Nodes(mask):
        mask = np.asarray(mask, bool)
        return Boundary(lambda mesh: mask.reshape(mesh.shape), "nodes")

    @staticmethod
    def side(name):
        return {"left": RectangularMesh2D.Left, "right": RectangularMesh2D.Right,
                "bottom": RectangularMesh2D.Bottom, "top": RectangularMesh2D.Top}[name]()


def wrap_symmetric(pts, sym, lows, highs=None):
    """Points as a provider reads them along axes where the geometry mirrors at 0
    (InterpolationFlags::wrap, plask/mesh/interpolation.hpp:232-250, non-periodic branch):
    a coordinate 0 becomes 1e-12, then, when the geometry lies on the positive side of the
    axis (its lower bound ``lows[d]`` >= 0), every coordinate reads at its absolute value,
    otherwise at minus it.  Returns the wrapped points and, per mirrored axis, the mask of
    points on the other side, whose vector components along that axis change sign
    (InterpolationFlags::postprocess, interpolation.hpp:272-287).  A mirrored axis whose
    geometry spans both sides of 0 (``lows[d]`` < 0 < ``highs[d]``) raises ValueError, as
    the reference's InterpolationFlags constructor does (interpolation.hpp:185-203)."""
    flips = {}
    if not any(sym):
        return pts, flips
    names = ("longitudinal", "transverse", "vertical") if len(sym) == 3 else ("horizontal", "vertical")
    for d, on in enumerate(sym):
        if on and highs is not None and lows[d] < 0.0 < highs[d]:
            raise ValueError(f"interpolation: Symmetric geometry spans at both sides of {names[d]} axis")
    w = np.array(pts, dtype=np.float64, copy=True)
    for d, on in enumerate(sym):
        if not on:
            continue
        x0 = w[:, d].copy()  # postprocess reflects on the coordinate as given
        x = np.where(x0 == 0.0, 1e-12, x0)
        if lows[d] >= 0.0:
            flips[d] = x0 < 0.0
            w[:, d] = np.abs(x)
        else:
            flips[d] = x0 > 0.0
            w[:, d] = -np.abs(x)
    return w, flips
