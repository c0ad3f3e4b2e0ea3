"""Solver configuration from PLaSK's XPL: the body of a ``<thermal>`` or ``<electrical>``
solver tag applied to the drop-in solver objects of this package.

What the reference reads there, and what this reader applies:

* ``Static3D``, ``Static2D``, ``StaticCyl`` (ThermalFem3DSolver::loadConfiguration,
  solvers/thermal/static/therm3d.cpp:40-69; therm2d.cpp:39-68): ``<temperature>``,
  ``<heatflux>``, ``<convection>``, ``<radiation>`` boundary conditions,
  ``<loop inittemp maxerr>``, ``<matrix algorithm>`` with ``<iterative ...>``
  (plask/common/fem/fem_solver.hpp:38-106), ``<mesh ref empty-elements>``
  (fem_solver.hpp:164-178), ``<geometry ref>``;
* ``Dynamic3D``, ``Dynamic2D``, ``DynamicCyl`` (solvers/thermal/dynamic/femT3d.cpp:46-70;
  femT2d.cpp:46-70): ``<temperature>``,
  ``<loop inittemp timestep rebuildfreq logfreq>``, ``<matrix methodparam lumping
  algorithm>``;
* ``Shockley3D`` (solvers/electrical/shockley/electr3d.cpp:41-87, beta.cpp:26-62):
  ``<voltage>``, ``<loop start-cond start-cond-inplane convergence maxerr>``,
  ``<contacts pcond ncond>``, ``<junction js beta beta<n> js<n>>``;
* ``ThermoElectric3D`` (solvers/meta/shockley/thermoelectric.py:94-172): ``<geometry
  thermal electrical>``, ``<mesh thermal electrical empty-elements>``, ``<junction pnjcond
  beta<n> js<n>>``, ``<contacts pcond ncond>``, ``<loop tfreq inittemp maxterr maxcerr>``,
  ``<tmatrix>`` / ``<ematrix>`` (algorithm, ``<iterative>``), the thermal conditions and
  ``<voltage>``.

A boundary condition is ``<condition place="SIDE" .../>`` (a side of the mesh:
``bottom``, ``top``, ``left``, ``right`` and in 3D ``back``, ``front``),
``<condition placeref="NAME" .../>`` (a place stored earlier under ``placename`` or
given in ``places``), or a nested ``<place side="SIDE"/>``
(plask/manager.hpp:704-736).  Values: ``value`` (temperature, heat flux, voltage),
``coeff`` and ``ambient`` (convection), ``emissivity`` and ``ambient`` (radiation).
Places defined by geometry objects need PLaSK's geometry tree, which this package
does not model; they are rejected with ``ValueError``.
"""
from __future__ import annotations

import logging
import xml.etree.ElementTree as ET

from .mesh import RectangularMesh2D, RectangularMesh3D

log = logging.getLogger("plask_gb300.xpl")

_ALGORITHMS = ("cholesky", "gauss", "iterative")
_EMPTY = ("default", "exclude", "include", "excluded", "included")
_ITER_ATTRS = {  # XPL attribute -> IterativeParams field (fem_solver.hpp:46-103)
    "accelerator": ("accelerator", str), "preconditioner": ("preconditioner", str), "noconv": ("noconv", str),
    "maxit": ("maxit", int), "maxerr": ("maxerr", float), "nfact": ("nfact", int), "omega": ("omega", float),
    "ndeg": ("ndeg", int), "lvfill": ("lvfill", int), "ltrunc": ("ltrunc", int), "nsave": ("ns1", int),
    "nrestart": ("ns2", int),
}


def _bool(text):
    t = text.strip().lower()
    if t in ("true", "yes", "1"):
        return True
    if t in ("false", "no", "0"):
        return False
    raise ValueError(f"not a boolean: {text!r}")


def _side(solver, name):
    mesh_cls = RectangularMesh2D if getattr(solver, "_geometry_kind", None) else RectangularMesh3D
    try:
        return mesh_cls.side(name.strip().lower())
    except KeyError:
        raise ValueError(f"unsupported boundary place {name!r}: only mesh sides are known here") from None


def _conditions(solver, tag, dest, kind, places):
    for cond in tag:
        if cond.tag != "condition":
            raise ValueError(f"unexpected <{cond.tag}> in <{tag.tag}>")
        a = cond.attrib
        if "place" in a:
            place = _side(solver, a["place"])
        elif "placeref" in a:
            if a["placeref"] not in places:
                raise ValueError(f"unknown boundary placeref {a['placeref']!r}")
            place = places[a["placeref"]]
        else:
            inner = [c for c in cond if c.tag == "place"]
            if len(inner) != 1:
                raise ValueError("a condition needs place, placeref or one <place> tag")
            pa = inner[0].attrib
            if "object" in pa or "side" not in pa:
                raise ValueError("places defined by geometry objects are not supported; use a mesh side")
            place = _side(solver, pa["side"])
        if "placename" in a:
            places[a["placename"]] = place
        if kind == "convection":
            value = {"coeff": float(a["coeff"]), "ambient": float(a["ambient"])}
        elif kind == "radiation":
            value = {"emissivity": float(a["emissivity"]), "ambient": float(a["ambient"])}
        else:
            value = float(a["value"])
        dest.append(place, value)


def _matrix(solver, tag):
    a = tag.attrib
    if "algorithm" in a:
        alg = a["algorithm"]
        if alg not in _ALGORITHMS:
            raise ValueError(f"unknown matrix algorithm {alg!r}")
        solver.algorithm = alg
    for sub in tag:
        if sub.tag != "iterative":
            raise ValueError(f"unexpected <{sub.tag}> in <matrix>")
        for k, v in sub.attrib.items():
            if k not in _ITER_ATTRS:
                raise ValueError(f"unexpected attribute {k!r} of <iterative>")
            field, conv = _ITER_ATTRS[k]
            setattr(solver.iterative, field, conv(v))


def _standard(solver, tag, geometries, meshes):
    """<geometry ref> and <mesh ref empty-elements> (Solver::parseStandardConfiguration)."""
    a = tag.attrib
    if tag.tag == "geometry":
        if "ref" in a:
            if a["ref"] not in geometries:
                raise ValueError(f"unknown geometry {a['ref']!r}")
            solver.geometry = geometries[a["ref"]]
        return
    if "ref" in a:
        if a["ref"] not in meshes:
            raise ValueError(f"unknown mesh {a['ref']!r}")
        solver.mesh = meshes[a["ref"]]
    if "empty-elements" in a:
        if a["empty-elements"] not in _EMPTY:
            raise ValueError(f"unknown empty-elements {a['empty-elements']!r}")
        solver.empty_elements = a["empty-elements"]


def _junction(solver, tag):
    for k, v in tag.attrib.items():
        if k == "js":
            solver.js = float(v)
        elif k == "beta":
            solver.beta = float(v)
        elif k == "pnjcond":
            log.warning("'pnjcond' attribute is obsolete; use <loop start-cond=>")
            solver.start_cond = float(v)
        elif k in ("wavelength", "heat"):
            continue
        elif k.startswith("beta") and k[4:].isdigit():
            setattr(solver, k, float(v))
        elif k.startswith("js") and k[2:].isdigit():
            setattr(solver, k, float(v))
        else:
            raise ValueError(f"unexpected attribute {k!r} of <junction>")


def _thermoelectric(te, root, places, geometries, meshes):
    """ThermoElectric._parse_xpl (thermoelectric.py:131-172) onto the two solvers."""
    th, el = te.thermal, te.electrical
    for tag in root:
        t, a = tag.tag, tag.attrib
        if t in ("geometry", "mesh"):
            table = geometries if t == "geometry" else meshes
            for key, solver in (("thermal", th), ("electrical", el)):
                if key in a:
                    if a[key] not in table:
                        raise ValueError(f"unknown {t} {a[key]!r}")
                    setattr(solver, t, table[a[key]])
            if t == "mesh" and "empty-elements" in a:
                if a["empty-elements"] not in _EMPTY:
                    raise ValueError(f"unknown empty-elements {a['empty-elements']!r}")
                el.empty_elements = a["empty-elements"]
        elif t == "junction":
            for k, v in a.items():
                if k == "pnjcond" or k.startswith("beta") or k.startswith("js"):
                    setattr(el, k, float(v))
        elif t == "contacts":
            for k in ("pcond", "ncond"):
                if k in a:
                    setattr(el, k, float(a[k]))
        elif t == "loop":
            te.tfreq = int(a.get("tfreq", te.tfreq))
            if "inittemp" in a:
                th.inittemp = float(a["inittemp"])
            if "maxterr" in a:
                th.maxerr = float(a["maxterr"])
            if "maxcerr" in a:
                el.maxerr = float(a["maxcerr"])
        elif t in ("tmatrix", "ematrix"):
            _matrix(th if t == "tmatrix" else el, tag)
        elif t in ("temperature", "heatflux", "convection", "radiation"):
            _conditions(th, tag, getattr(th, f"{t}_boundary"), t, places)
        elif t == "voltage":
            _conditions(el, tag, el.voltage_boundary, "voltage", places)
        else:
            raise ValueError(f"unexpected <{t}> in the configuration of ThermoElectric3D")
    return te


def configure(solver, xml, places=None, geometries=None, meshes=None):
    """Apply the XPL configuration ``xml`` (the solver tag or its body, as text or an
    ElementTree element) to ``solver``.  ``places``, ``geometries`` and ``meshes`` map the
    names that ``placeref`` and ``ref`` attributes use; ``placename`` adds to ``places``."""
    root = ET.fromstring(xml) if isinstance(xml, str) else xml
    places = {} if places is None else places
    geometries = geometries or {}
    meshes = meshes or {}
    cls = type(solver).__name__
    if hasattr(solver, "thermal") and hasattr(solver, "electrical"):
        return _thermoelectric(solver, root, places, geometries, meshes)
    electrical = hasattr(solver, "voltage_boundary")
    dynamic = cls in ("Dynamic3D", "Dynamic2D", "DynamicCyl")
    for tag in root:
        t, a = tag.tag, tag.attrib
        if t in ("geometry", "mesh"):
            _standard(solver, tag, geometries, meshes)
        elif t == "matrix":
            if dynamic:
                if "methodparam" in a:
                    solver.methodparam = float(a["methodparam"])
                if "lumping" in a:
                    solver.lumping = _bool(a["lumping"])
                rest = ET.Element("matrix", {k: v for k, v in a.items() if k not in ("methodparam", "lumping")})
                rest.extend(list(tag))
                tag = rest
            _matrix(solver, tag)
        elif electrical and t == "voltage":
            _conditions(solver, tag, solver.voltage_boundary, "voltage", places)
        elif electrical and t == "loop":
            if "start-cond" in a or "start-cond-inplane" in a:
                c0, c1 = solver.start_cond
                if "start-cond" in a:
                    parts = a["start-cond"].split(",")
                    if len(parts) == 2:
                        if "start-cond-inplane" in a:
                            raise ValueError("'start-cond' has two values and 'start-cond-inplane' is also given")
                        c0, c1 = float(parts[0]), float(parts[1])
                    else:
                        c1 = float(parts[0])
                c0 = float(a.get("start-cond-inplane", c0))
                solver.start_cond = (c0, c1)
            if "convergence" in a:
                solver.convergence = a["convergence"]
            if "maxerr" in a:
                solver.maxerr = float(a["maxerr"])
        elif electrical and t == "contacts":
            if "pcond" in a:
                solver.pcond = float(a["pcond"])
            if "ncond" in a:
                solver.ncond = float(a["ncond"])
        elif electrical and t == "junction":
            _junction(solver, tag)
        elif not electrical and t == "loop":
            names = ("inittemp", "timestep", "rebuildfreq", "logfreq") if dynamic else ("inittemp", "maxerr")
            for k, v in a.items():
                if k not in names:
                    raise ValueError(f"unexpected attribute {k!r} of <loop>")
                setattr(solver, k, int(v) if k in ("rebuildfreq", "logfreq") else float(v))
        elif not electrical and t in ("temperature", "heatflux", "convection", "radiation"):
            dest = getattr(solver, f"{t}_boundary")
            if dynamic and t != "temperature":
                raise ValueError(f"{cls} takes temperature boundary conditions only")
            _conditions(solver, tag, dest, t, places)
        else:
            raise ValueError(f"unexpected <{t}> in the configuration of {cls}")
    return solver
