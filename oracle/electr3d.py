"""CPU oracle for the Shockley3D FEM core -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of PLaSK's ``electrical.shockley.Shockley3D``
(solvers/electrical/shockley/electr3d.cpp, beta.hpp), sharing the mesh
numbering and linear solves of oracle/fem3d.py:

* ``active_regions``    setupActiveRegions                   electr3d.cpp:94-184
* ``junction_update``   junction conductivity update          electr3d.cpp:246-274, beta.hpp:43-46
* ``assemble``          setMatrix (no load vector)            electr3d.cpp:276-344
* ``currents``          current density and error             electr3d.cpp:389-424
* ``compute``           the loop                               electr3d.cpp:356-442
* ``heat``              saveHeatDensity                        electr3d.cpp:444-478
* ``total_current``     integrateCurrent / getTotalCurrent    electr3d.cpp:480-505
* ``total_heat``        getTotalHeat                           electr3d.cpp:612-624

Element conductivities are (c00, c11) = (in-plane, vertical) in S/m.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.sparse as sp

from . import fem3d as F


@dataclasses.dataclass
class ElecProblem:
    """Shockley3D problem.  cond: (ne2, ne1, ne0, 2) conductivities of non-junction
    elements; junction: (ne2, ne1, ne0) int, region number + 1 or 0; empty: element
    mask of EMPTY material; voltage: [(node mask, V)]; beta/js per region."""

    axes: tuple
    cond: np.ndarray
    junction: np.ndarray
    beta: list
    js: list
    voltage: list
    empty: np.ndarray | None = None
    order: str = "012"
    maxerr: float = 0.05
    convergence: str = "fast"
    start_cond: tuple = (0.0, 5.0)
    empty_elements: str = "exclude"
    temperature: np.ndarray | None = None  # element temperature read by beta(T), js(T)

    @property
    def shape(self):
        return tuple(len(a) for a in self.axes[::-1])

    def as_problem(self):
        """A thermal Problem with the same mesh, masking and Dirichlet sets (for numbering and BCs)."""
        mat = np.zeros(self.junction.shape, np.int32)
        empty = np.zeros(2, bool)
        if self.empty is not None:
            mat[self.empty] = 1
            empty[1] = True
        mats = F.Materials(np.ones(2), np.zeros(2), empty=empty)
        return F.Problem(axes=self.axes, mat=mat, materials=mats, heat=np.zeros(mat.shape), temperature=self.voltage,
                         order=self.order, empty_elements=self.empty_elements)


def active_regions(prob: ElecProblem):
    """Per region: (bottom, top) node-plane indices and height (electr3d.cpp:94-184)."""
    z = np.asarray(prob.axes[2], np.float64)
    out = []
    for reg in range(1, int(prob.junction.max(initial=0)) + 1):
        ks = np.nonzero(np.any(prob.junction == reg, axis=(1, 2)))[0]
        if ks.size == 0:
            continue
        bottom, top = int(ks.min()), int(ks.max()) + 1
        cols = prob.junction[ks.min()] == reg
        for k in ks:
            if not np.array_equal(prob.junction[k] == reg, cols):
                raise ValueError(f"junction {reg - 1} does not have top and bottom edges at constant heights")
        out.append((bottom, top, z[top] - z[bottom]))
    return out


def initial_conds(prob: ElecProblem):
    """loadConductivity (electr3d.cpp:203-225) with the default junction conductivity."""
    c = np.array(prob.cond, np.float64, copy=True)
    j = prob.junction > 0
    c[j, 0] = prob.start_cond[0]
    c[j, 1] = prob.start_cond[1]
    small = j & (np.isnan(c[..., 1]) | (np.abs(c[..., 1]) < 1e-16))
    c[small, 1] = 1e-16
    return c


def junction_update(prob: ElecProblem, conds, V):
    """New conductivities of junction elements from the potential (electr3d.cpp:246-274).

    V: full-grid potential (n2, n1, n0)."""
    regs = active_regions(prob)
    c = conds.copy()
    for reg, (bot, top, h) in enumerate(regs, start=1):
        kk, jj, ii = np.nonzero(prob.junction == reg)
        U = 0.25 * (-V[bot, jj, ii] - V[bot, jj, ii + 1] - V[bot, jj + 1, ii] - V[bot, jj + 1, ii + 1]
                    + V[top, jj, ii] + V[top, jj, ii + 1] + V[top, jj + 1, ii] + V[top, jj + 1, ii + 1])
        jy = 0.1 * c[kk, jj, ii, 1] * U / h
        jy = np.abs(jy)
        beta, js = prob.beta[reg - 1], prob.js[reg - 1]
        if callable(beta):  # beta(T), js(T) of the Python solver (electr_python.cpp:104-111)
            beta = np.array([beta(t) for t in prob.temperature[kk, jj, ii]])
        if callable(js):
            js = np.array([js(t) for t in prob.temperature[kk, jj, ii]])
        new11 = 10.0 * jy * beta * h / np.log(1e7 * jy / js + 1.0)
        new00 = np.zeros_like(new11)
        if prob.convergence == "stable":
            new00 = 0.5 * (c[kk, jj, ii, 0] + new00)
            new11 = 0.5 * (c[kk, jj, ii, 1] + new11)
        bad = np.isnan(new11) | (np.abs(new11) < 1e-16)
        new11[bad] = 1e-16
        c[kk, jj, ii, 0] = new00
        c[kk, jj, ii, 1] = new11
    return c


def assemble(prob: ElecProblem, conds, numbering):
    """Stiffness matrix of setMatrix (electr3d.cpp:276-344): K_e of therm3d with (c00, c11)."""
    node_id, n_active = numbering
    tp = prob.as_problem()
    act = F.element_active(tp).ravel()
    shape = prob.shape
    n2, n1, n0 = shape
    nodes_c = F._element_nodes(shape)[:, act]
    ids = node_id.ravel()[nodes_c]
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    ne = (n2 - 1, n1 - 1, n0 - 1)
    kk, jj, ii = (a.ravel()[act] for a in np.meshgrid(*(np.arange(m) for m in ne), indexing="ij"))
    dx, dy, dz = x0[ii + 1] - x0[ii], x1[jj + 1] - x1[jj], x2[kk + 1] - x2[kk]
    c = conds.reshape(-1, 2)[act]
    ky = c[:, 0] * 1e-6
    kz = c[:, 1] * 1e-6
    kx = ky.copy()
    kx = kx / dx; kx = kx * dy; kx = kx * dz
    ky = ky * dx; ky = ky / dy; ky = ky * dz
    kz = kz * dx; kz = kz * dy; kz = kz / dz
    g = {0: (kx + ky + kz) / 9.0, 1: (-2.0 * kx + ky + kz) / 18.0, 2: (kx - 2.0 * ky + kz) / 18.0,
         4: (kx + ky - 2.0 * kz) / 18.0, 6: (kx - 2.0 * ky - 2.0 * kz) / 36.0, 5: (-2.0 * kx + ky - 2.0 * kz) / 36.0,
         3: (-2.0 * kx - 2.0 * ky + kz) / 36.0, 7: -(kx + ky + kz) / 36.0}
    rows, cols, data = [], [], []
    for a in range(8):
        for b in range(a + 1):
            v = g[a ^ b]
            rows.append(ids[a]); cols.append(ids[b]); data.append(v)
            if a != b:
                rows.append(ids[b]); cols.append(ids[a]); data.append(v)
    return sp.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))), shape=(n_active, n_active))


def _grad_terms(prob, V):
    shape = prob.shape
    nodes = F._element_nodes(shape)
    t = V.ravel()[nodes]
    lll, ull, lul, uul, llu, ulu, luu, uuu = t
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    ne = tuple(s - 1 for s in shape)
    kk, jj, ii = (a.ravel() for a in np.meshgrid(*(np.arange(m) for m in ne), indexing="ij"))
    sx = (-lll - llu - lul - luu + ull + ulu + uul + uuu) / (x0[ii + 1] - x0[ii])
    sy = (-lll - llu + lul + luu - ull - ulu + uul + uuu) / (x1[jj + 1] - x1[jj])
    sz = (-lll + llu - lul + luu - ull + ulu - uul + uuu) / (x2[kk + 1] - x2[kk])
    return sx, sy, sz


def currents(prob: ElecProblem, V, conds):
    """Current density [kA/cm2] per element (electr3d.cpp:389-414), shape (ne2, ne1, ne0, 3)."""
    sx, sy, sz = _grad_terms(prob, V)
    c = conds.reshape(-1, 2)
    j = np.stack([-0.025 * c[:, 0] * sx, -0.025 * c[:, 0] * sy, -0.025 * c[:, 1] * sz], axis=-1)
    return j.reshape(prob.junction.shape + (3,))


def heat(prob: ElecProblem, V, conds):
    """Joule heat density [W/m3] per element (electr3d.cpp:444-478); zero in empty elements."""
    sx, sy, sz = _grad_terms(prob, V)
    dvx, dvy, dvz = -0.25e6 * sx, -0.25e6 * sy, -0.25e6 * sz
    c = conds.reshape(-1, 2)
    h = c[:, 0] * dvx * dvx + c[:, 0] * dvy * dvy + c[:, 1] * dvz * dvz
    h = h.reshape(prob.junction.shape)
    if prob.empty is not None:
        h[prob.empty] = 0.0
    return h


def total_current(prob: ElecProblem, V, conds, region=0):
    """Current through the middle plane of a junction [mA] (electr3d.cpp:480-505)."""
    bot, top, _ = active_regions(prob)[region]
    level = (bot + top) // 2
    j = currents(prob, V, conds)
    x0, x1 = (np.asarray(a, np.float64) for a in prob.axes[:2])
    area = np.diff(x1)[:, None] * np.diff(x0)[None, :]
    sel = prob.junction[level] > 0
    return float(np.sum(j[level, :, :, 2][sel] * area[sel]) * 0.01)


def total_heat(prob: ElecProblem, V, conds):
    """Total Joule heat [mW] (electr3d.cpp:612-624)."""
    h = heat(prob, V, conds)
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    vol = np.diff(x2)[:, None, None] * np.diff(x1)[None, :, None] * np.diff(x0)[None, None, :]
    tp = prob.as_problem()
    act = F.element_active(tp)
    return float(np.sum((1e-15 * vol * h)[act]))


def compute(prob: ElecProblem, loops=0, V=None, conds=None, loopno=0, method="cholesky", state=None):
    """ElectricalFem3DSolver::compute (electr3d.cpp:356-442).

    Returns (V, conds, toterr, records) with records of (loop, max |j| at the junction, err %).
    ``state`` (a dict) carries V, conds, the current density and loopno from one call to
    the next, as the solver object does between compute() calls."""
    if state is not None and state:
        V, conds, loopno = state["V"], state["conds"], state["loopno"]
    tp = prob.as_problem()
    numbering = F.masked_numbering(tp)
    node_id, n = numbering
    if V is None:
        V = np.zeros(prob.shape)
    if conds is None:
        conds = initial_conds(prob)
    is_d, vf, vl = F.dirichlet_values(tp, node_id, n)
    noactive = not np.any(prob.junction > 0)
    minj = 100e-7
    current = np.zeros(prob.junction.shape + (3,))
    if state is not None and "current" in state:
        current = state["current"]
    act_el = F.element_active(tp)
    toterr, loop, records = 0.0, 0, []
    while True:
        if loopno != 0:
            conds = junction_update(prob, conds, V)
        A = assemble(prob, conds, numbering)
        A2, b = F.apply_dirichlet(A, np.zeros(n), is_d, vf, vl)
        x = F.solve(A2, b, method)
        V = F.to_full(tp, node_id, x, fill=0.0)
        cur = currents(prob, V, conds)
        sel = act_el & ((prob.junction > 0) if not noactive else True)
        a2 = np.sum(cur * cur, axis=-1)
        mcur = float(np.sqrt(np.max(a2[sel]))) if np.any(sel) else 0.0
        d2 = np.sum((current - cur) ** 2, axis=-1)
        err = float(np.max(d2[act_el])) if np.any(act_el) else 0.0
        err = 100.0 * np.sqrt(err) / max(mcur, minj)
        if (loop != 0 or mcur >= minj) and err > toterr:
            toterr = err
        current = cur
        loopno += 1
        loop += 1
        records.append((loop, mcur, err))
        if not (err > prob.maxerr and (loops == 0 or loop < loops)):
            break
    if state is not None:
        state.update(V=V, conds=conds, current=current, loopno=loopno)
    return V, conds, toterr, records


def from_structure(s, order="012", convergence="fast", empty_elements="exclude", maxerr=None):
    """ElecProblem of a structure generator's output (plask_gb300.structures.ElecStructure)."""
    empty = s.empty[s.mat] if np.any(s.empty) else None
    return ElecProblem(axes=tuple(np.asarray(a, np.float64) for a in s.axes), cond=s.element_cond(),
                       junction=np.asarray(s.junction), beta=list(s.beta), js=list(s.js),
                       voltage=[(np.asarray(m, bool), float(v)) for m, v in s.voltage], empty=empty, order=order,
                       maxerr=s.maxerr if maxerr is None else maxerr, convergence=convergence,
                       empty_elements=empty_elements)


def total_energy(prob: ElecProblem, V, eps_elem):
    """Electrostatic energy [J] (electr3d.cpp:567-599); eps_elem: relative permittivity per element."""
    sx, sy, sz = _grad_terms(prob, V)
    dvx, dvy, dvz = -0.25e6 * sx, -0.25e6 * sy, -0.25e6 * sz
    w = np.asarray(eps_elem, np.float64).ravel() * (dvx * dvx + dvy * dvy + dvz * dvz)
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    vol = (np.diff(x2)[:, None, None] * np.diff(x1)[None, :, None] * np.diff(x0)[None, None, :]).ravel()
    act = F.element_active(prob.as_problem()).ravel()
    epsilon0 = 1.0 / (4e-7 * np.pi) / 299792458.0 / 299792458.0  # plask/phys/constants.hpp:32-35
    return float(np.sum((0.5e-18 * epsilon0 * vol * w)[act]))
