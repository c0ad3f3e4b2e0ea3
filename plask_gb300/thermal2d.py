"""``Static2D`` and ``StaticCyl``: the 2D finite-element thermal solvers, on the GPU.

Drop-ins for PLaSK's ``thermal.static.Static2D`` and ``thermal.static.StaticCyl``
(solvers/thermal/static/therm2d.hpp:27-118, therm2d.cpp, python/therm_python.cpp:102-125):
the same attribute names, defaults, boundary-condition lists, receiver and providers as
:class:`plask_gb300.thermal.Static3D`, on a :class:`RectangularMesh2D`.  The
computation runs in ``libplgpu_fem3d.so`` (a planar handle, include/plgpu_fem2d.h).

Geometry: ``geometry`` is any object with ``materials`` (a :class:`MaterialTable`;
``kz_ratio`` is the vertical/horizontal ratio) and ``material_ids(mesh)`` returning one
material id per element, canonical shape (n1-1, n0-1), e.g. :class:`StructureGeometry2D`.
In StaticCyl axis 0 is the radius.
"""
from __future__ import annotations

import logging

import numpy as np

from . import _native
from .mesh import RectangularMesh2D, mesh_index2d, to_mesh_order2d, wrap_symmetric
from .thermal import (BadInput, BoundaryConditions, IterativeParams, MaterialTable, Provider, _check_interpolation,
                      _element_axis, _nearest_axis, conductivity_elements, load_state, masked_element_interpolate,
                      masked_interpolate, save_state, spline_interpolate)

log = logging.getLogger("plask_gb300.thermal2d")


class StructureGeometry2D:
    """Geometry given as element material ids on a fixed mesh, or a callable of midpoints (x, y).

    ``symmetric``: per axis, whether the geometry is mirrored at 0 (a ``mirror`` edge,
    plask/geometry/space.hpp:147-150); the cylindrical solvers mirror r in any case."""

    def __init__(self, materials: MaterialTable, mat=None, material_at=None, leaf_height=None,
                 symmetric=(False, False)):
        self.materials = materials
        self._mat = None if mat is None else np.asarray(mat, np.int32)
        self._at = material_at
        self._leaf = leaf_height
        self.symmetric = tuple(bool(v) for v in symmetric)

    def material_ids(self, mesh: RectangularMesh2D):
        if self._mat is not None:
            if self._mat.shape != mesh.element_shape:
                raise BadInput(-1, f"material ids of shape {self._mat.shape} do not fit the mesh {mesh.element_shape}")
            return self._mat
        if self._at is None:
            raise BadInput(-1, "geometry has neither material ids nor a material function")
        mids = mesh.element_midpoints()
        return np.asarray(self._at(mids[..., 0], mids[..., 1]), np.int32)

    def leaf_height(self, mesh):
        return None if self._leaf is None else np.asarray(self._leaf, np.float64)

    @classmethod
    def from_structure(cls, s):
        return cls(MaterialTable(s.k300, s.p, s.kz_ratio, s.hexp, s.empty, tables=getattr(s, "ktables", None)),
                   mat=s.mat)


class Receiver2D:
    """``inHeat``: heat density [W/m^3]; a constant, an element array (n1-1, n0-1), or a callable of (x, y)."""

    def __init__(self, owner, default=0.0):
        self._owner = owner
        self._value = default

    def attach(self, value):
        self._value = value
        self._owner._heat_changed()

    def __call__(self, mesh: RectangularMesh2D):
        v = self._value
        if callable(v) and not isinstance(v, np.ndarray):
            mids = mesh.element_midpoints()
            return np.broadcast_to(np.asarray(v(mids[..., 0], mids[..., 1]), np.float64), mesh.element_shape)
        return np.broadcast_to(np.asarray(v, np.float64), mesh.element_shape)


def _points2d(dst):
    if isinstance(dst, RectangularMesh2D):
        Y, X = np.meshgrid(dst.axis1, dst.axis0, indexing="ij")
        pts = np.stack([X, Y], axis=-1).reshape(-1, 2)
        out = np.empty_like(pts)
        out[dst.index_array().ravel()] = pts
        return out
    return np.asarray(dst, np.float64).reshape(-1, 2)


def _bilinear(axes, F, pts, fill, box=None):
    """Bilinear interpolation of canonical F (n1, n0) at points (m, 2); outside the axes
    the edge values continue (plask/mesh/axis1d.cpp:99-154), or ``fill`` (unless None)
    outside the axes (``box``)."""
    ii, ww, ok = [], [], np.ones(len(pts), bool)
    for d in range(2):
        a = axes[d]
        x = pts[:, d]
        i = np.clip(np.searchsorted(a, x, side="right") - 1, 0, a.size - 2)
        w = np.clip((x - a[i]) / (a[i + 1] - a[i]), 0.0, 1.0)
        b = a if box is None else box[d]
        ok &= (x >= b[0]) & (x <= b[-1])
        ii.append(i)
        ww.append(w)
    out = np.zeros(len(pts))
    for cj in (0, 1):
        for ci in (0, 1):
            wt = (ww[0] if ci else 1 - ww[0]) * (ww[1] if cj else 1 - ww[1])
            out += wt * F[np.minimum(ii[1] + cj, F.shape[0] - 1), np.minimum(ii[0] + ci, F.shape[1] - 1)]
    if fill is not None:
        out[~ok] = fill
    return out


class Static2D:
    """Finite element thermal solver for 2D Cartesian geometry, computed on the GPU.

    Attributes (therm2d.hpp:27-118, therm_python.cpp:102-118, fem/python.hpp:31-41):
    ``geometry``, ``mesh`` (:class:`RectangularMesh2D`), ``inittemp`` (300 K), ``maxerr``
    (0.05 K), ``algorithm`` ("iterative"; also "cholesky", "gauss", "gpu-pcg",
    "gpu-mixed"), ``iterative``, ``empty_elements``, the four boundary-condition lists,
    ``inHeat``/``inHeatDensity`` and the providers ``outTemperature``, ``outHeatFlux``,
    ``outThermalConductivity``.  GPU knobs as in Static3D: ``rtol``, ``residual_norm``,
    ``bc_compat`` (True: the reference's convective edge stiffness).
    """

    _geometry_kind = "cartesian"
    _class_name = "thermal.Static2D"

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
        self._inHeat = Receiver2D(self)
        self.outTemperature = Provider(self._get_temperatures)
        self.outHeatFlux = Provider(self._get_heat_fluxes)
        self.outThermalConductivity = Provider(self._get_conductivity)
        self._fem = None
        self._elements_dirty = self._bc_dirty = self._heat_dirty = True
        self._toterr = 0.0
        self.stats = {}
        self.loop_log = []

    @property
    def id(self):
        return f"{self.name}:{self._class_name}" if self.name else self._class_name

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
        if not isinstance(m, RectangularMesh2D):
            raise BadInput(-1, f"{self.id}: the mesh must be a RectangularMesh2D")
        self._mesh = m
        self.invalidate()
        self._fem = None

    @property
    def algorithm(self):
        return self._algorithm

    @algorithm.setter
    def algorithm(self, a):
        if a not in _native.ALGORITHMS or a == "gpu-learned":
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
    def inHeat(self):
        return self._inHeat

    @inHeat.setter
    def inHeat(self, v):
        self._inHeat.attach(v)

    inHeatDensity = inHeat

    @property
    def err(self):
        """Maximum estimated error of the last compute() (therm2d.hpp:101)."""
        return self._toterr

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
            self._fem = _native.Fem2D(self._mesh.axes, self._mesh.ordering, self._geometry_kind)
            self._fem.set_log_callback(self._log)
            self._elements_dirty = self._bc_dirty = self._heat_dirty = True
        fem = self._fem
        order = self._mesh.ordering
        if self._elements_dirty:
            mt = self._geometry.materials
            fem.set_materials(mt.k300, mt.p, mt.kz_ratio, mt.hexp, mt.empty)
            mt.apply_tables(fem)
            mat = self._geometry.material_ids(self._mesh)
            leaf = self._geometry.leaf_height(self._mesh)
            fem.set_elements(to_mesh_order2d(mat, order), to_mesh_order2d(self._inHeat(self._mesh), order),
                             None if leaf is None else to_mesh_order2d(leaf, order))
            self._elements_dirty = self._heat_dirty = False
        elif self._heat_dirty:
            fem.set_heat(to_mesh_order2d(self._inHeat(self._mesh), order))
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
        """Forget the computed temperatures (therm2d.cpp:117-121)."""
        if self._fem is not None:
            self._fem.invalidate()
        self._elements_dirty = True

    def _log(self, level, msg):
        if msg.startswith("Loop "):
            self.loop_log.append(msg)
        lvl = {2: logging.WARNING, 3: logging.INFO, 4: logging.INFO}.get(level, logging.DEBUG)
        log.log(lvl, "%s: %s", self.id, msg)

    def compute(self, loops=0):
        """Run thermal calculations; returns the maximum temperature correction (therm2d.cpp:444-502)."""
        self.initialize()
        self.loop_log = []
        tot, st = self._fem.compute(loops)
        self._toterr = tot
        self.stats = st
        self.iterative.converged = bool(st["converged"])
        self.iterative.iters = st["inner_iterations"]
        self.iterative.err = st["last_rel_residual"]
        return tot

    # ------------------------------------------------------------------ results
    def temperatures(self):
        """Nodal temperatures in the solver's numbering (masked mesh, mesh order)."""
        self.initialize()
        return self._fem.temperature()

    def save(self, path):
        """Checkpoint the temperature field to an ``.npz`` file (thermal.save_state)."""
        save_state(self, path)

    def load(self, path):
        """Start the next ``compute()`` from a checkpointed field (thermal.load_state)."""
        load_state(self, path)

    def _active_elements(self):
        """Canonical mask of the masked mesh's elements (fem_solver.hpp:164-189)."""
        mat = self._geometry.material_ids(self._mesh)
        mt = self._geometry.materials
        excl = self._empty_elements in ("exclude", "excluded") or (
            self._empty_elements == "default" and self._algorithm != "iterative")
        return ~mt.empty[mat] if excl else np.ones(mat.shape, bool)

    def _active_mask_mesh_order(self):
        mesh = self._mesh
        act = self._active_elements()
        n1, n0 = mesh.shape
        used = np.zeros(mesh.shape, bool)
        for cj in (0, 1):
            for ci in (0, 1):
                used[cj:n1 - 1 + cj, ci:n0 - 1 + ci] |= act
        return to_mesh_order2d(used, mesh.ordering)

    def _full_temperature(self):
        """Canonical (n1, n0) temperature with NaN at nodes outside the masked mesh."""
        t = self._fem.temperature()
        n = len(self._mesh)
        idx = self._mesh.index_array().ravel()
        if t.size == n:
            return t[idx].reshape(self._mesh.shape)
        vals = np.full(n, np.nan)
        vals[np.flatnonzero(self._active_mask_mesh_order())] = t
        return vals[idx].reshape(self._mesh.shape)

    def _wrap(self, pts):
        """Points as the providers see them (InterpolationFlags::wrap,
        plask/mesh/interpolation.hpp:232-250): along an axis the geometry mirrors at 0 -- r in
        the cylindrical geometry always (plask/geometry/space.hpp:1068-1072) -- a negative
        coordinate reads at its absolute value.  Returns the wrapped points and, per mirrored
        axis, the mask of reflected points (their normal vector components change sign,
        InterpolationFlags::postprocess, interpolation.hpp:272-287)."""
        sym = list(getattr(self._geometry, "symmetric", (False, False)) or (False, False)) + [False, False]
        sym = sym[:2]
        if self._geometry_kind == "cylindrical":
            sym[0] = True
        if not any(sym):
            return pts, {}
        return wrap_symmetric(pts, sym, [float(a[0]) for a in self._mesh.axes], [float(a[-1]) for a in self._mesh.axes])

    def _get_temperatures(self, dst_mesh, interpolation="linear"):
        """Temperatures on a destination mesh or points (therm2d.cpp:544-553): bilinear or the
        nearest node, the edge values continuing outside the mesh; on a masked mesh its
        element search, 300 K where no included element holds the point."""
        if self._fem is None:
            n = len(dst_mesh) if dst_mesh is not None else 0
            return np.full(n, self.inittemp)
        T = self._full_temperature()
        if dst_mesh is None:
            return T
        pts, _ = self._wrap(_points2d(dst_mesh))
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
            i0, i1 = (_nearest_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            out = T[i1, i0]
            return np.where(np.isnan(out), 300.0, out)
        return _bilinear(self._mesh.axes, T, pts, fill=None)

    def heat_fluxes(self):
        """Per-element heat flux [W/m^2], canonical (ne1, ne0, 2) (saveHeatFluxes)."""
        self.initialize()
        q = self._fem.heat_flux()
        eidx = self._mesh.element_index_array().ravel()
        return q[eidx].reshape(self._mesh.element_shape + (2,))

    def _get_heat_fluxes(self, dst_mesh, interpolation="linear"):
        """Heat flux at points (therm2d.cpp:556-571): bilinear over the element midpoints or the
        holding element, the edge values continuing outside; on a masked mesh its element
        mesh's interpolation, 0 where no included element holds the point."""
        if self._fem is None:
            n = len(dst_mesh) if dst_mesh is not None else 0
            return np.zeros((n, 2))
        q = np.nan_to_num(self.heat_fluxes())
        if dst_mesh is None:
            return q
        mids = [0.5 * (a[1:] + a[:-1]) for a in self._mesh.axes]
        pts, flips = self._wrap(_points2d(dst_mesh))
        active = self._active_elements()
        method = _check_interpolation(interpolation, splines=True)
        if method in ("spline", "smooth_spline"):
            if not np.all(active):
                raise BadInput(-1, f"{self.id}: spline interpolation of heat fluxes on a masked mesh is not provided")
            out = np.stack([spline_interpolate(mids, q[..., c], pts, method) for c in range(2)], axis=-1)
        elif not np.all(active):
            # the masked element mesh's interpolation; NaN reads 0 (SafeData)
            out = np.nan_to_num(masked_element_interpolate(self._mesh.axes, q, active, pts, method))
        elif method == "nearest":
            i0, i1 = (_element_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            out = q[i1, i0].copy()
        else:
            out = np.stack([_bilinear(mids, q[..., c], pts, fill=None) for c in range(2)], axis=-1)
        for d, m in flips.items():  # the normal component of a mirrored point (Symmetry NP / PN)
            out[m, d] *= -1.0
        return out

    def _get_conductivity(self, dst_mesh, interpolation="linear"):
        """(k_0, k_1) of the element holding each point (therm2d.cpp:574-597), NaN outside."""
        self.initialize()
        k = self._fem.conductivity()
        eidx = self._mesh.element_index_array().ravel()
        k = k[eidx].reshape(self._mesh.element_shape + (2,))
        if dst_mesh is None:
            return k
        idx, ok = conductivity_elements(self._mesh.axes, self._wrap(_points2d(dst_mesh))[0])
        out = k[idx[1], idx[0]].copy()
        out[~ok] = np.nan
        return out

    def thickness(self):
        """Layer-run thickness per element, canonical (ne1, ne0) (therm2d.cpp:81-114)."""
        self.initialize()
        th = self._fem.thickness()
        eidx = self._mesh.element_index_array().ravel()
        return th[eidx].reshape(self._mesh.element_shape)


class StaticCyl(Static2D):
    """Finite element thermal solver for 2D cylindrical geometry (axis 0 = r >= 0), on the GPU
    (ThermalFem2DSolver<Geometry2DCylindrical>, therm2d.cpp:301-441; therm_python.cpp:119-125)."""

    _geometry_kind = "cylindrical"
    _class_name = "thermal.StaticCyl"


class Dynamic2D(Static2D):
    """Finite element time-stepping thermal solver for 2D Cartesian geometry, on the GPU.

    A drop-in for PLaSK's ``thermal.dynamic.Dynamic2D`` (femT2d.cpp,
    python/dynamic_python.cpp:32-69): ``compute(time)`` advances ``time`` ns with the theta
    method; attributes ``inittemp`` (300 K), ``timestep`` (0.1 ns), ``methodparam`` (0.5:
    Crank-Nicolson), ``lumping`` (True: lumped heat capacity; False: the consistent matrix
    c (4, 2, 1) / 9, femT2d.cpp:199-233), ``rebuildfreq`` (0), ``logfreq`` (500),
    ``time`` / ``elapsed_time`` (read only), ``temperature_boundary``, ``inHeat`` and the
    providers of Static2D.  The material table must carry ``cp`` and ``dens``.
    """

    _class_name = "thermal.Dynamic2D"

    def __init__(self, name=""):
        super().__init__(name)
        self.timestep = 0.1
        self.methodparam = 0.5
        self.lumping = True
        self.rebuildfreq = 0
        self.logfreq = 500
        self._elapstime = 0.0
        # the time-stepping solvers have temperature conditions only (femT2d.cpp:48-70)
        del self.heatflux_boundary, self.convection_boundary, self.radiation_boundary
        self.heatflux_boundary = self.convection_boundary = self.radiation_boundary = ()

    @property
    def time(self):
        """Time of calculations performed so far since the last invalidation [ns]."""
        return self._elapstime

    elapsed_time = time

    def compute(self, time):
        """Run thermal calculations for ``time`` ns (femT2d.cpp:387-445)."""
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


class DynamicCyl(Dynamic2D):
    """Finite element time-stepping thermal solver for 2D cylindrical geometry (axis 0 = r),
    on the GPU (DynamicThermalFem2DSolver<Geometry2DCylindrical>, femT2d.cpp:256-384)."""

    _geometry_kind = "cylindrical"
    _class_name = "thermal.DynamicCyl"


def solver_for_structure2d(s, cls=Static2D, ordering="best", algorithm="gpu-mixed", name="", **kw):
    """A configured :class:`Static2D` / :class:`StaticCyl` (or, with their temperature
    conditions only, :class:`Dynamic2D` / :class:`DynamicCyl`) for a generated 2D structure."""
    mesh = RectangularMesh2D(*s.axes, ordering=ordering)
    sv = cls(name)
    sv.geometry = StructureGeometry2D.from_structure(s)
    sv.mesh = mesh
    sv.inHeat = s.heat
    sv.inittemp = s.inittemp
    sv.maxerr = s.maxerr
    sv.algorithm = algorithm
    for side, v in s.temperature:
        sv.temperature_boundary.append(RectangularMesh2D.side(side), v)
    if not issubclass(cls, Dynamic2D):
        for side, v in s.heatflux:
            sv.heatflux_boundary.append(RectangularMesh2D.side(side), v)
        for side, h, ta in s.convection:
            sv.convection_boundary.append(RectangularMesh2D.side(side), {"coeff": h, "ambient": ta})
        for side, e, ta in s.radiation:
            sv.radiation_boundary.append(RectangularMesh2D.side(side), {"emissivity": e, "ambient": ta})
    for k, v in kw.items():
        setattr(sv, k, v)
    return sv


__all__ = ["Static2D", "StaticCyl", "Dynamic2D", "DynamicCyl", "StructureGeometry2D", "RectangularMesh2D", "solver_for_structure2d",
           "mesh_index2d"]
