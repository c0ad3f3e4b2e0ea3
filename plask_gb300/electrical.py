"""``Shockley3D`` and ``ThermoElectric3D``: the 3D electrical FEM solver and the
thermo-electric loop, on the GPU.

``Shockley3D`` is a drop-in for PLaSK's ``electrical.shockley.Shockley3D``
(solvers/electrical/shockley/electr3d.hpp, electr3d.cpp, beta.hpp,
python/electr_python.cpp:31-115, 180-262): the same attribute names and defaults
(``beta``/``js`` with ``beta<n>``/``js<n>`` per junction, numbers or functions of
the temperature; ``maxerr`` 0.05 %, ``convergence``, ``pcond``/``ncond``,
``start_cond``, ``algorithm`` "iterative", ``empty_elements``), the
``voltage_boundary`` list, the ``inTemperature`` receiver and the ``outVoltage``,
``outCurrentDensity``, ``outHeat`` and ``outConductivity`` providers, and
``get_total_current``, ``get_total_heat``, ``get_electrostatic_energy`` and
``get_capacitance``.  The computation runs in ``libplgpu_fem3d.so``
(include/plgpu_elec3d.h); this module converts inputs and outputs.

``ThermoElectric3D`` follows solvers/meta/shockley/thermoelectric.py:69-220: the
electrical solver runs ``tfreq`` loops, the thermal solver one, until both errors
are below their ``maxerr``.  With both solvers on the same mesh the Joule heat
moves from the electrical to the thermal handle on the device.

Geometry: an :class:`ElecGeometry` gives per-element material ids, junction
numbers and contact roles on a fixed mesh (PLaSK asks its geometry tree for the
material and roles at every element midpoint).
"""
from __future__ import annotations

import dataclasses
import logging
import pathlib
import sys
import time

import numpy as np

from . import _native
from .mesh import RectangularMesh3D, to_mesh_order, wrap_symmetric
from .thermal import BadInput, BoundaryConditions, ComputationError, IterativeParams, Provider, Static3D
from .thermal import (_check_interpolation, _element_axis, _nearest_axis, _points, _trilinear,
                      masked_element_interpolate, masked_interpolate, spline_interpolate)

log = logging.getLogger("plask_gb300.electrical")

__all__ = ["ElecMaterialTable", "ElecGeometry", "Shockley3D", "ThermoElectric3D", "ComputationError", "BadInput"]


@dataclasses.dataclass
class ElecMaterialTable:
    """Per-material electrical data: conductivity tensor (S/m), relative permittivity,
    EMPTY kind and the "noheat" role.  ``cond_T`` (optional) maps (material ids, T) to
    (c00, c11) arrays for temperature-dependent materials (Material::cond(T))."""

    cond_xy: np.ndarray
    cond_z: np.ndarray
    eps: np.ndarray | None = None
    empty: np.ndarray | None = None
    noheat: np.ndarray | None = None
    cond_T: object = None

    def __post_init__(self):
        self.cond_xy = np.asarray(self.cond_xy, np.float64)
        n = self.cond_xy.size
        self.cond_z = np.asarray(self.cond_z, np.float64)
        self.eps = np.ones(n) if self.eps is None else np.asarray(self.eps, np.float64)
        self.empty = np.zeros(n, bool) if self.empty is None else np.asarray(self.empty, bool)
        self.noheat = np.zeros(n, bool) if self.noheat is None else np.asarray(self.noheat, bool)


class ElecGeometry:
    """Element material ids, junction numbers (0 outside, n + 1 in junction n) and contact
    roles (0 none, 1 "p-contact", 2 "n-contact") on a fixed mesh."""

    def __init__(self, materials: ElecMaterialTable, mat, junction=None, contacts=None, symmetric=(False, False)):
        self.materials = materials
        self._mat = np.asarray(mat, np.int32)
        self._junc = np.zeros(self._mat.shape, np.int32) if junction is None else np.asarray(junction, np.int32)
        self._contacts = None if contacts is None else np.asarray(contacts, np.int8)
        self.symmetric = tuple(bool(s) for s in symmetric)

    def _fit(self, a, mesh, what):
        if a.shape != mesh.element_shape:
            raise BadInput(-1, f"{what} of shape {a.shape} do not fit the mesh {mesh.element_shape}")
        return a

    def material_ids(self, mesh):
        return self._fit(self._mat, mesh, "material ids")

    def junction_ids(self, mesh):
        return self._fit(self._junc, mesh, "junction numbers")

    def contact_roles(self, mesh):
        return None if self._contacts is None else self._fit(self._contacts, mesh, "contact roles")

    @classmethod
    def from_structure(cls, s):
        return cls(ElecMaterialTable(s.cond_xy, s.cond_z, s.eps, s.empty, s.noheat), s.mat, s.junction,
                   symmetric=s.symmetric)


class TemperatureReceiver:
    """``inTemperature``: a constant (300 K by default), a canonical element array, a
    Static3D solver (its element-average temperatures) or a callable of midpoints."""

    def __init__(self, owner, default=300.0):
        self._owner = owner
        self._value = default

    def attach(self, value):
        self._value = value
        self._owner._temperature_changed()

    @property
    def value(self):
        return self._value

    def __call__(self, mesh):
        v = self._value
        if isinstance(v, Static3D):
            if v._fem is None:
                return np.full(mesh.element_shape, v.inittemp)
            if all(np.array_equal(a, b) for a, b in zip(v._mesh.axes, mesh.axes)):
                t = _native.element_temperature(v._fem)  # element averages on the device
                eidx = v._mesh.element_index_array().ravel()
                return t[eidx].reshape(v._mesh.element_shape)
            pts = mesh.element_midpoints().reshape(-1, 3)
            return v._get_temperatures(pts).reshape(mesh.element_shape)  # the thermal provider
        if isinstance(v, Provider):
            mids = mesh.element_midpoints().reshape(-1, 3)
            return np.asarray(v(mids), np.float64).reshape(mesh.element_shape)
        if callable(v) and not isinstance(v, np.ndarray):
            mids = mesh.element_midpoints()
            return np.broadcast_to(np.asarray(v(mids[..., 0], mids[..., 1], mids[..., 2]), np.float64),
                                   mesh.element_shape)
        return np.broadcast_to(np.asarray(v, np.float64), mesh.element_shape)


class Shockley3D:
    """Finite element electrical solver for 3D geometry with Shockley junctions, on the GPU."""

    def __init__(self, name=""):
        object.__setattr__(self, "_beta", [float("nan")])  # BetaSolver(name), beta.cpp:18-22
        object.__setattr__(self, "_js", [1.0])
        self.name = name
        self._geometry = None
        self._mesh = None
        self.maxerr = 0.05
        self._convergence = "fast"
        self.pcond = 5.0
        self.ncond = 50.0
        self._start_cond = (0.0, 5.0)
        self._algorithm = "iterative"
        self.iterative = IterativeParams()
        self._empty_elements = "default"
        self.rtol = 1e-14
        self.voltage_boundary = BoundaryConditions(self, _native.BC_TEMPERATURE, 1)
        self._inTemperature = TemperatureReceiver(self)
        self.outVoltage = Provider(self._get_voltage)
        self.outCurrentDensity = Provider(self._get_current_density)
        self.outHeat = Provider(self._get_heat)
        self.outConductivity = Provider(self._get_conductivity)
        self._elec = None
        self._elements_dirty = True
        self._bc_dirty = True
        self._temperature_dirty = True
        self._computed = False
        self._toterr = 0.0
        self.stats = {}
        self.loop_log = []

    # ---------------------------------------------------------------- beta / js
    def _set_param(self, lst, n, value, default):
        if n < 0:
            raise BadInput(-1, "junction number must be >= 0")
        if not (callable(value) or np.isscalar(value)):
            raise TypeError(f"{self.id}: parameter {n} must be a float or a callable")
        while len(lst) <= n:
            lst.append(default)
        lst[n] = value if callable(value) else float(value)
        object.__setattr__(self, "_junc_dirty", True)
        self.invalidate()

    def _get_param(self, lst, n, what):
        if n >= len(lst):
            raise BadInput(-1, f"{self.id}: no {what} given for junction {n}")
        return lst[n]

    @property
    def beta(self):
        """Junction coefficient of junction 0 (1/V): a number or a function of T."""
        return self._get_param(self._beta, 0, "beta")

    @beta.setter
    def beta(self, v):
        self._set_param(self._beta, 0, v, float("nan"))

    @property
    def js(self):
        """Reverse bias current density of junction 0 (A/m^2): a number or a function of T."""
        return self._get_param(self._js, 0, "js")

    @js.setter
    def js(self, v):
        self._set_param(self._js, 0, v, 1.0)

    def __getattr__(self, attr):
        for pre, lst in (("beta", "_beta"), ("js", "_js")):
            if attr.startswith(pre) and attr[len(pre):].isdigit():
                return self._get_param(object.__getattribute__(self, lst), int(attr[len(pre):]), pre)
        raise AttributeError(f"'Shockley3D' object has no attribute '{attr}'")

    def __setattr__(self, attr, value):
        for pre, lst, dflt in (("beta", "_beta", float("nan")), ("js", "_js", 1.0)):
            if attr.startswith(pre) and attr[len(pre):].isdigit():
                self._set_param(object.__getattribute__(self, lst), int(attr[len(pre):]), value, dflt)
                return
        object.__setattr__(self, attr, value)

    # ---------------------------------------------------------------- properties
    @property
    def id(self):
        return f"{self.name}:electrical.Shockley3D" if self.name else "electrical.Shockley3D"

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
        self._elec = None

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
    def convergence(self):
        return self._convergence

    @convergence.setter
    def convergence(self, v):
        if v not in ("fast", "stable"):
            raise BadInput(-1, f"unknown convergence {v!r}")
        self._convergence = v

    @property
    def start_cond(self):
        """Junction conductivity before the first update (electr_python.cpp:216-221)."""
        return self._start_cond

    @start_cond.setter
    def start_cond(self, v):
        self._start_cond = (0.0, float(v)) if np.isscalar(v) else tuple(float(c) for c in v)
        if self._elec is not None:
            c = (float(v), float(v)) if np.isscalar(v) else self._start_cond  # setCondJunc(double), electr3d.hpp:267-270
            self._elec.set_junction_conductivity(*c)

    pnjcond = start_cond

    @property
    def inTemperature(self):
        return self._inTemperature

    @inTemperature.setter
    def inTemperature(self, v):
        self._inTemperature.attach(v)

    @property
    def err(self):
        return self._toterr

    # ---------------------------------------------------------------- lifecycle
    def _bc_changed(self):
        self._bc_dirty = True

    def _temperature_changed(self):
        self._temperature_dirty = True

    def _needs_temperature(self):
        mt = self._geometry.materials
        return (mt.cond_T is not None or any(callable(b) for b in self._beta) or any(callable(j) for j in self._js))

    def initialize(self):
        if self._geometry is None:
            raise BadInput(-1, f"{self.id}: No geometry specified")
        if self._mesh is None:
            raise BadInput(-1, f"{self.id}: No mesh specified")
        if self._elec is None:
            self._elec = _native.Elec3D(self._mesh.axes, self._mesh.ordering)
            self._elements_dirty = self._bc_dirty = self._temperature_dirty = True
            object.__setattr__(self, "_junc_dirty", True)
        el = self._elec
        order = self._mesh.ordering
        if self._elements_dirty:
            mt = self._geometry.materials
            el.set_materials(mt.cond_xy, mt.cond_z, mt.eps, mt.empty, mt.noheat)
            el.set_elements(to_mesh_order(self._geometry.material_ids(self._mesh), order),
                            to_mesh_order(self._geometry.junction_ids(self._mesh), order))
            c = self._start_cond
            el.set_junction_conductivity(*c)
            self._elements_dirty = False
            self._temperature_dirty = True
        if self._bc_dirty:
            el.clear_voltage()
            for place, vals in self.voltage_boundary:
                nodes = place.nodes(self._mesh) if hasattr(place, "nodes") else np.asarray(place, np.int64)
                el.add_voltage(nodes, vals[0])
            self._bc_dirty = False
        if getattr(self, "_junc_dirty", True):
            nj = max(len(self._beta), len(self._js))
            for n in range(nj):
                b = self._beta[n] if n < len(self._beta) else float("nan")
                j = self._js[n] if n < len(self._js) else 1.0
                el.set_junction(n, float("nan") if callable(b) else b, 1.0 if callable(j) else j)
            object.__setattr__(self, "_junc_dirty", False)
        it = self.iterative
        maxit = it.maxit if self._algorithm == "iterative" and it.maxit != 1000 else 0
        el.set_solver(self._algorithm, self.rtol, maxit, it.noconv, self._empty_elements)
        el.set_loop(self.maxerr, self._convergence)

    def _load_conductivity(self):
        """loadConductivity's host part (electr3d.cpp:203-225): temperature-dependent
        materials, contact roles and beta(T)/js(T) evaluated at the element temperatures."""
        mesh, geo, el = self._mesh, self._geometry, self._elec
        order = mesh.ordering
        mt = geo.materials
        roles = geo.contact_roles(mesh)
        T = self._inTemperature(mesh) if self._needs_temperature() else None
        if mt.cond_T is not None or roles is not None:
            mat = geo.material_ids(mesh)
            over = np.full(mesh.element_shape + (2,), np.nan)
            if mt.cond_T is not None:
                c00, c11 = mt.cond_T(mat, T)
                over[..., 0] = c00
                over[..., 1] = c11
            if roles is not None:
                over[roles == 1] = self.pcond
                over[roles == 2] = self.ncond
            el.set_element_conductivity(to_mesh_order(over, order))
        else:
            el.set_element_conductivity(None)
        if any(callable(b) for b in self._beta) or any(callable(j) for j in self._js):
            junc = geo.junction_ids(mesh)
            bj = np.full(mesh.element_shape + (2,), np.nan)
            for n in range(int(junc.max(initial=0))):
                sel = junc == n + 1
                if not np.any(sel):
                    continue
                # activeCond reads the temperature of the junction's middle layer (electr3d.cpp:258-259)
                ks = np.nonzero(np.any(sel, axis=(1, 2)))[0]
                mid = (int(ks.min()) + int(ks.max()) + 1) // 2
                Tm = np.broadcast_to(T[mid], T.shape)[sel]
                b = self._get_param(self._beta, n, "beta")
                j = self._get_param(self._js, n, "js")
                bj[sel, 0] = np.array([b(t) for t in Tm]) if callable(b) else b
                bj[sel, 1] = np.array([j(t) for t in Tm]) if callable(j) else j
            el.set_junction_params(to_mesh_order(bj, order))
        else:
            el.set_junction_params(None)
        self._temperature_dirty = False

    def invalidate(self):
        """onInvalidate (electr3d.cpp:195-201)."""
        if getattr(self, "_elec", None) is not None:
            self._elec.invalidate()
            c = self._start_cond
            self._elec.set_junction_conductivity(*c)
        self._computed = False

    # ---------------------------------------------------------------- computation
    def compute(self, loops=0):
        """Run electrical calculations; returns the maximum current-density error [%]."""
        self.initialize()
        self._load_conductivity()
        tot, st = self._elec.compute(loops)
        self._toterr = tot
        self.stats = st
        self._computed = True
        self.iterative.converged = bool(st["converged"])
        self.iterative.iters = st["inner_iterations"]
        self.iterative.err = st["last_rel_residual"]
        return tot

    def _sym(self):
        s = self._geometry.symmetric
        return (2.0 if s[0] else 1.0) * (2.0 if s[1] else 1.0)

    def get_total_current(self, nact=0):
        """Total current through the middle of junction ``nact`` [mA] (electr3d.cpp:480-505)."""
        return self._elec.total_current(nact) * self._sym()

    def get_total_heat(self):
        """Total Joule heat [mW] (electr3d.cpp:612-624)."""
        return self._elec.total_heat() * self._sym()

    def get_electrostatic_energy(self):
        """Energy of the electrostatic field [J] (electr3d.cpp:567-599)."""
        return self._elec.total_energy()

    def get_capacitance(self):
        """2 W / U^2 [pF] with U the difference of the two voltage conditions (electr3d.cpp:601-610)."""
        return self._elec.capacitance()

    # ---------------------------------------------------------------- results
    def _full_potential(self):
        """Canonical (n2, n1, n0) potential with NaN outside the masked mesh."""
        mesh = self._mesh
        nn = self._node_count()
        v = self._elec.potential(nn)
        canon_idx = mesh.index_array().ravel()
        if nn == len(mesh):
            return v[canon_idx].reshape(mesh.shape)
        act = self._active_mask_mesh_order()
        vals = np.full(len(mesh), np.nan)
        vals[np.flatnonzero(act)] = v
        return vals[canon_idx].reshape(mesh.shape)

    def _excluding(self):
        return self._empty_elements in ("exclude", "excluded") or (
            self._empty_elements == "default" and self._algorithm != "iterative")

    def _active_mask_mesh_order(self):
        mesh = self._mesh
        mat = self._geometry.material_ids(mesh)
        mt = self._geometry.materials
        act_el = ~mt.empty[mat] if self._excluding() else np.ones(mat.shape, bool)
        n2, n1, n0 = mesh.shape
        used = np.zeros(mesh.shape, bool)
        for ck in (0, 1):
            for cj in (0, 1):
                for ci in (0, 1):
                    used[ck:n2 - 1 + ck, cj:n1 - 1 + cj, ci:n0 - 1 + ci] |= act_el
        return to_mesh_order(used, mesh.ordering)

    def _node_count(self):
        if not self._excluding():
            return len(self._mesh)
        mt = self._geometry.materials
        if not np.any(mt.empty[self._geometry.material_ids(self._mesh)]):
            return len(self._mesh)
        return int(self._active_mask_mesh_order().sum())

    def _element_field(self, flat, comps=None):
        eidx = self._mesh.element_index_array().ravel()
        shp = self._mesh.element_shape + (() if comps is None else (comps,))
        return flat[eidx].reshape(shp)

    def current_densities(self):
        """Per-element current density [kA/cm^2], canonical (ne2, ne1, ne0, 3)."""
        return self._element_field(self._elec.current_density(), 3)

    def heat_densities(self):
        """Per-element Joule heat [W/m^3], canonical (ne2, ne1, ne0) (saveHeatDensity)."""
        return self._element_field(self._elec.heat())

    def conductivities(self):
        """Per-element (c00, c11) [S/m], canonical (ne2, ne1, ne0, 2) (getConductivity)."""
        self.initialize()
        self._load_conductivity()
        return self._element_field(self._elec.conductivity(), 2)

    def _wrap(self, pts):
        """Points as the providers see them (InterpolationFlags::wrap,
        plask/mesh/interpolation.hpp:232-250): along an axis mirrored at 0 (the structure's
        ``symmetric`` flags) a negative coordinate reads at its absolute value.  Returns the
        wrapped points and, per mirrored axis, the mask of reflected points."""
        sym = tuple(getattr(self._geometry, "symmetric", ())) if self._geometry is not None else ()
        if not any(sym):
            return pts, {}
        return wrap_symmetric(pts, sym, [float(a[0]) for a in self._mesh.axes], [float(a[-1]) for a in self._mesh.axes])

    def _get_voltage(self, dst_mesh, interpolation="linear"):
        """Potential on a destination mesh (electr3d.cpp:507-515): trilinear or the nearest
        node, the edge values continuing outside the mesh; on a masked mesh its element
        search, NaN where no included element holds the point."""
        V = self._full_potential()
        if dst_mesh is None:
            return V
        pts, _ = self._wrap(_points(dst_mesh))
        method = _check_interpolation(interpolation, splines=True)
        active = self._active_elements()
        masked = not np.all(active)
        if method in ("spline", "smooth_spline"):
            return spline_interpolate(self._mesh.axes, V, pts, method, active if masked else None)
        if masked:
            return masked_interpolate(self._mesh.axes, V, active, pts, method)
        if method == "nearest":
            i0, i1, i2 = (_nearest_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            return V[i2, i1, i0]
        return _trilinear(self._mesh.axes, V, pts, fill=None)

    def _element_interp(self, q, dst_mesh=None, pts=None, interpolation="linear"):
        """Element values at points, 0 outside (electr3d.cpp:517-555): over the element
        midpoints, or the holding element; on a masked mesh the masked element mesh's
        interpolation with NaN read as 0."""
        mids = [0.5 * (a[1:] + a[:-1]) for a in self._mesh.axes]
        pts, flips = self._wrap(_points(dst_mesh) if pts is None else pts)
        out = self._element_values(q, mids, pts, interpolation)
        if q.ndim == 4:
            for d, m in flips.items():  # the normal component of a mirrored point (Symmetry NPP / PNP)
                out[m, d] *= -1.0
        return out

    def _element_values(self, q, mids, pts, interpolation):
        method = _check_interpolation(interpolation)
        active = self._active_elements()
        if not np.all(active):
            return np.nan_to_num(masked_element_interpolate(self._mesh.axes, q, active, pts, method))
        if method == "nearest":
            i0, i1, i2 = (_element_axis(a, pts[:, d]) for d, a in enumerate(self._mesh.axes))
            out = q[i2, i1, i0].copy()
            inside = np.all([(pts[:, d] >= a[0]) & (pts[:, d] <= a[-1]) for d, a in enumerate(self._mesh.axes)], axis=0)
            out[~inside] = 0.0
            return out
        if q.ndim == 3:
            return _trilinear(mids, q, pts, fill=0.0, clamp=True, box=self._mesh.axes)
        return np.stack([_trilinear(mids, q[..., c], pts, fill=0.0, clamp=True, box=self._mesh.axes)
                         for c in range(q.shape[-1])], axis=-1)

    def _get_current_density(self, dst_mesh, interpolation="linear"):
        """Current density on a destination mesh (electr3d.cpp:517-535): 0 outside."""
        j = np.nan_to_num(self.current_densities())
        return j if dst_mesh is None else self._element_interp(j, dst_mesh, interpolation=interpolation)

    def _get_heat(self, dst_mesh, interpolation="linear"):
        """Heat density on a destination mesh (electr3d.cpp:537-555): 0 outside."""
        h = np.nan_to_num(self.heat_densities())
        return h if dst_mesh is None else self._element_interp(h, dst_mesh, interpolation=interpolation)

    def _active_elements(self):
        mat = self._geometry.material_ids(self._mesh)
        return ~self._geometry.materials.empty[mat] if self._excluding() else np.ones(mat.shape, bool)

    def _get_conductivity(self, dst_mesh, interpolation="nearest"):
        """Conductivity of the element holding each point (electr3d.cpp:557-565): the masked
        element mesh's nearest lookup, NaN where no included element holds the point."""
        c = self.conductivities()
        if dst_mesh is None:
            return c
        return masked_element_interpolate(self._mesh.axes, c, self._active_elements(), self._wrap(_points(dst_mesh))[0],
                                          "nearest")


class ThermoElectric3D:
    """Self-consistent thermo-electric loop (solvers/meta/shockley/thermoelectric.py:69-220).

    ``thermal`` (Static3D) and ``electrical`` (Shockley3D) are created here and
    connected: the electrical solver reads the thermal temperatures, the thermal
    solver the Joule heat.  ``compute`` alternates ``electrical.compute(tfreq)`` and
    ``thermal.compute(1)`` until both return errors within their ``maxerr``.
    ``save`` writes the fields the reference saves to HDF5 (thermoelectric.py:259-290) to
    an ``.npz`` file instead (no HDF5 library here), and only on request: ``compute``'s
    ``save`` defaults to False."""

    # the solvers' providers (thermoelectric.py:651-670)
    outTemperature = property(lambda self: self.thermal.outTemperature)
    outHeatFlux = property(lambda self: self.thermal.outHeatFlux)
    outThermalConductivity = property(lambda self: self.thermal.outThermalConductivity)
    outVoltage = property(lambda self: self.electrical.outVoltage)
    outCurrentDensity = property(lambda self: self.electrical.outCurrentDensity)
    outHeat = property(lambda self: self.electrical.outHeat)
    outConductivity = property(lambda self: self.electrical.outConductivity)

    def __init__(self, name=""):
        self.name = name
        self.thermal = Static3D(name)
        self.electrical = Shockley3D(name)
        self.tfreq = 6
        self.history = []
        self.reconnect()

    def reconnect(self):
        self.electrical.inTemperature = self.thermal

    def initialize(self):
        self.thermal.initialize()
        self.electrical.initialize()

    def invalidate(self):
        self.thermal.invalidate()
        self.electrical.invalidate()

    def _same_mesh(self):
        a, b = self.thermal.mesh, self.electrical.mesh
        return all(np.array_equal(x, y) for x, y in zip(a.axes, b.axes))

    def _move_heat(self):
        if self._same_mesh():
            _native.heat_from(self.thermal._fem, self.electrical._elec)  # device to device
        else:
            tm = self.thermal.mesh
            pts = tm.element_midpoints().reshape(-1, 3)
            q = self.electrical._element_interp(np.nan_to_num(self.electrical.heat_densities()), pts=pts)
            self.thermal.inHeat = q.reshape(tm.element_shape)

    def compute(self, save=False, invalidate=True, group="ThermoElectric"):
        """Run the loop (thermoelectric.py:181-219); ``save`` (True or a file name) writes the
        fields afterwards (:meth:`save`)."""
        if invalidate:
            self.invalidate()
        self.initialize()
        verr = 2.0 * self.electrical.maxerr
        terr = 2.0 * self.thermal.maxerr
        self.history = []
        while terr > self.thermal.maxerr or verr > self.electrical.maxerr:
            verr = self.electrical.compute(self.tfreq)
            self._move_heat()
            terr = self.thermal.compute(1)
            self.history.append((verr, terr))
        if save:
            self.save(None if save is True else save, group)
        return verr, terr

    def get_temperature(self):
        """Temperature on the thermal mesh, in its order (thermoelectric.py:292-296)."""
        return self.thermal.outTemperature(self.thermal.mesh)

    def get_voltage(self):
        """Potential on the electrical mesh, in its order (thermoelectric.py:298-302)."""
        return self.electrical.outVoltage(self.electrical.mesh)

    def get_vertical_voltage(self, at=0):
        """Potential along the vertical axis at horizontal position ``at`` (a number for
        both horizontal axes, or a pair) on the electrical mesh's vertical nodes
        (thermoelectric.py:304-322)."""
        try:
            at0, at1 = at
        except TypeError:
            at0 = at1 = at
        z = np.asarray(self.electrical.mesh.axis2, np.float64)
        pts = np.stack([np.full(z.size, float(at0)), np.full(z.size, float(at1)), z], axis=1)
        return self.electrical.outVoltage(pts)

    def save(self, filename=None, group="ThermoElectric"):
        """Write the temperature on the thermal mesh, the potential on the electrical mesh and
        the current density of the electrical elements (the fields of
        thermoelectric.py:259-271) to the ``.npz`` file ``filename`` under the keys
        ``<group>/Temperature``, ``<group>/Potential``, ``<group>/CurrentDensity``, each with
        its mesh axes (``.../axis0`` ...) and iteration order (``.../ordering``); canonical
        array shapes (axis 0 last).  Without ``filename`` the name is the script's with the
        current time.  Returns the file name."""
        if filename is None:
            stem = pathlib.Path(sys.argv[0]).stem if sys.argv and sys.argv[0] else "plask"
            filename = f"{stem or 'plask'}-{time.strftime('%Y%m%d-%H%M%S')}.npz"
        tm, vm = self.thermal.mesh, self.electrical.mesh

        def canonical(values, mesh):
            # provider values come in the mesh's order; index_array maps canonical to mesh order
            return np.asarray(values)[mesh.index_array().ravel()].reshape(mesh.shape)

        data = {f"{group}/Temperature": canonical(self.get_temperature(), tm),
                f"{group}/Potential": canonical(self.get_voltage(), vm),
                f"{group}/CurrentDensity": np.asarray(self.electrical.outCurrentDensity(None))}
        for key, mesh, mids in ((f"{group}/Temperature", tm, False), (f"{group}/Potential", vm, False),
                                (f"{group}/CurrentDensity", vm, True)):
            for d, a in enumerate(mesh.axes):
                a = np.asarray(a, np.float64)
                data[f"{key}/axis{d}"] = 0.5 * (a[1:] + a[:-1]) if mids else a
            data[f"{key}/ordering"] = np.array(mesh.ordering)
        np.savez(filename, **data)
        log.info("Fields saved to file '%s' in group '%s'", filename, group)
        return str(filename)

    def get_total_current(self, nact=0):
        return self.electrical.get_total_current(nact)


def solver_for_structure(s, ordering="best", algorithm="gpu-mixed", name="", **kw):
    """A configured :class:`Shockley3D` for a generated structure (plask_gb300.structures.ElecStructure)."""
    mesh = RectangularMesh3D(*s.axes, ordering=ordering)
    sv = Shockley3D(name)
    sv.geometry = ElecGeometry.from_structure(s)
    sv.mesh = mesh
    sv.maxerr = s.maxerr
    sv.algorithm = algorithm
    for n, (b, j) in enumerate(zip(s.beta, s.js)):
        setattr(sv, f"beta{n}", b)
        setattr(sv, f"js{n}", j)
    for m, v in s.voltage:
        sv.voltage_boundary.append(RectangularMesh3D.Nodes(m), v)
    for k, v in kw.items():
        setattr(sv, k, v)
    return sv
