"""CPU oracle for the 2D FEM thermal solvers (Static2D, StaticCyl) -- TEST INFRASTRUCTURE ONLY.

Only tests, the smoke check and the benchmark's CPU-baseline leg may import this
module; the product path never calls it.

It restates, in FP64 numpy, what PLaSK's ``thermal.static.Static2D`` and
``thermal.static.StaticCyl`` (``ThermalFem2DSolver<Geometry2DCartesian>`` and
``<Geometry2DCylindrical>``) do for one ``compute()`` call, citing the reference
lines it follows (paths relative to the PLaSK source tree):

* ``element_thickness``   solvers/thermal/static/therm2d.cpp:81-114
* ``masked_numbering``    plask/mesh/rectangular_masked2d.cpp (nodes of non-empty
                          elements in the full mesh's iteration order),
                          plask/mesh/rectangular2d.cpp:20-50 (ORDER_10 / ORDER_01)
* ``assemble``            solvers/thermal/static/therm2d.cpp:139-172 (setBoundaries),
                          :176-299 (Cartesian setMatrix), :301-441 (cylindrical)
* Dirichlet elimination   plask/common/fem/matrix.hpp:111-145 (oracle/fem3d.py)
* ``compute``             solvers/thermal/static/therm2d.cpp:444-502
* ``heat_fluxes``         solvers/thermal/static/therm2d.cpp:505-541

Two properties of the reference's edge terms are reproduced when ``bc_compat`` is
True (the default): the convective stiffness (coeff_1 + coeff_2) len / 6 and / 12
has no micrometre factor while its load term has 0.5e-6 (therm2d.cpp:242-255,
367-392), and in the cylindrical form the edge stiffness is multiplied by the
element's midpoint radius a second time when the element matrix r K_e is added
(therm2d.cpp:410-420).  With ``bc_compat=False`` the stiffness gets 1e-6 len and one
radius weight, consistent with the load term.

Array conventions: node arrays have shape ``(n1, n0)`` (axis 0 fastest), element
arrays ``(n1-1, n0-1)``; axis 1 is vertical; in the cylindrical form axis 0 is the
radius.  Lengths in micrometres, heat densities in W/m^3, conductivities in W/(m K).
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.sparse as sp

from . import fem3d as F3

SB = F3.SB


@dataclasses.dataclass
class Problem2D:
    """One Static2D / StaticCyl problem.  Boundary places are boolean node masks (n1, n0).

    * ``temperature``: [(mask, T)];  ``heatflux``: [(mask, q)];
    * ``convection``: [(mask, h, T_amb)];  ``radiation``: [(mask, eps, T_amb)]
    """

    axes: tuple
    mat: np.ndarray
    materials: F3.Materials
    heat: np.ndarray
    geometry: str = "cartesian"  # or "cylindrical"
    temperature: list = dataclasses.field(default_factory=list)
    heatflux: list = dataclasses.field(default_factory=list)
    convection: list = dataclasses.field(default_factory=list)
    radiation: list = dataclasses.field(default_factory=list)
    order: str = "01"
    inittemp: float = 300.0
    maxerr: float = 0.05
    empty_elements: str = "exclude"
    bc_compat: bool = True

    @property
    def shape(self):
        return (len(self.axes[1]), len(self.axes[0]))  # (n1, n0)


def reference_order(shape, order):
    """Mesh index of every node: ORDER_01 index = i1 + n1 i0, ORDER_10 index = i0 + n0 i1."""
    n1, n0 = shape
    j, i = np.meshgrid(np.arange(n1), np.arange(n0), indexing="ij")
    if order == "01":
        return (j + n1 * i).astype(np.int64)
    if order == "10":
        return (i + n0 * j).astype(np.int64)
    raise ValueError(order)


def element_active(prob):
    if prob.empty_elements == "include":
        return np.ones(prob.mat.shape, bool)
    return ~prob.materials.empty[prob.mat]


def masked_numbering(prob):
    """(node_id (n1, n0) with -1 for dropped nodes, n_active), masked ids in mesh order."""
    act = element_active(prob)
    n1, n0 = prob.shape
    used = np.zeros((n1, n0), bool)
    for cj in (0, 1):
        for ci in (0, 1):
            used[cj:n1 - 1 + cj, ci:n0 - 1 + ci] |= act
    ref = reference_order(prob.shape, prob.order)
    flat = np.flatnonzero(used.ravel())
    order = np.argsort(ref.ravel()[flat], kind="stable")
    ids = np.empty(flat.size, np.int64)
    ids[order] = np.arange(flat.size)
    node_id = np.full((n1, n0), -1, np.int64)
    node_id.ravel()[flat] = ids
    return node_id, int(flat.size)


def element_thickness(prob):
    """Height of the maximal same-material run along axis 1 (therm2d.cpp:81-114)."""
    mat = prob.mat
    y = np.asarray(prob.axes[1], np.float64)
    th = np.empty(mat.shape)
    ne1, ne0 = mat.shape
    for i in range(ne0):
        start = 0
        for j in range(1, ne1 + 1):
            if j == ne1 or mat[j, i] != mat[j - 1, i]:
                th[start:j, i] = y[j] - y[start]
                start = j
    return th


def _corners(shape):
    """Canonical node index of corners (LL, LR, UL, UR) of every element, (4, ne)."""
    n1, n0 = shape
    jj, ii = np.meshgrid(np.arange(n1 - 1), np.arange(n0 - 1), indexing="ij")
    base = (ii + n0 * jj).ravel()
    return np.stack([base, base + 1, base + n0, base + n0 + 1])


def first_match(conds, shape, nvals):
    """Per node: whether a condition applies and the values of the first one listing it."""
    has = np.zeros(shape, bool).ravel()
    vals = np.zeros((nvals,) + shape).reshape(nvals, -1)
    for c in conds:
        m = np.asarray(c[0], bool).ravel() & ~has
        for k in range(nvals):
            vals[k, m] = c[1 + k]
        has |= m
    return has, vals


def assemble(prob, T, thickness=None, numbering=None):
    """Stiffness matrix and load vector before Dirichlet elimination (therm2d.cpp:176-299, 301-441).

    ``T`` is the nodal temperature on the full grid (n1, n0).  Returns (A, F) over the
    masked numbering."""
    n1, n0 = prob.shape
    node_id, n_act = numbering if numbering is not None else masked_numbering(prob)
    if thickness is None:
        thickness = element_thickness(prob)
    cyl = prob.geometry == "cylindrical"
    x0, x1 = (np.asarray(a, np.float64) for a in prob.axes)
    Tf = np.asarray(T, np.float64).ravel()
    corners = _corners(prob.shape)
    act = element_active(prob).ravel()
    jj, ii = (a.ravel() for a in np.meshgrid(np.arange(n1 - 1), np.arange(n0 - 1), indexing="ij"))
    rows, cols, data = [], [], []
    Fv = np.zeros(n_act)
    bc = {
        "hf": first_match(prob.heatflux, prob.shape, 1),
        "cv": first_match(prob.convection, prob.shape, 2),
        "rd": first_match(prob.radiation, prob.shape, 2),
    }
    kscale = 1.0 if prob.bc_compat else 1e-6
    matv = prob.mat.ravel()
    heat = prob.heat.ravel()
    th = np.asarray(thickness).ravel()
    for e in np.flatnonzero(act):
        i, j = int(ii[e]), int(jj[e])
        ll, lr, ul, ur = (int(c) for c in corners[:, e])
        nodes = (ll, lr, ur, ul)  # setBoundaries' i1..i4
        w = x0[i + 1] - x0[i]
        h = x1[j + 1] - x1[j]
        r = 0.5 * (x0[i] + x0[i + 1])
        temp = 0.25 * (Tf[ll] + Tf[lr] + Tf[ul] + Tf[ur])
        kx, ky = prob.materials.thermk(np.array([matv[e]]), np.array([temp]), np.array([th[e]]))
        kx, ky = float(kx[0]), float(ky[0])
        if cyl:
            kx = kx * h / w
            ky = ky * w / h
            f = 0.25e-12 * r * w * h * heat[e]
        else:
            kx *= h
            kx /= w
            ky *= w
            ky /= h
            f = 0.25e-12 * w * h * heat[e]
        # element matrix over (i1..i4) = (ll, lr, ur, ul): conduction and edge terms apart
        Kc = np.zeros((4, 4))
        Kc[0, 0] = Kc[1, 1] = Kc[2, 2] = Kc[3, 3] = (kx + ky) / 3.0
        Kc[3, 2] = Kc[2, 3] = Kc[1, 0] = Kc[0, 1] = (-2.0 * kx + ky) / 6.0   # k43, k21
        Kc[3, 1] = Kc[1, 3] = Kc[2, 0] = Kc[0, 2] = -(kx + ky) / 6.0         # k42, k31
        Kc[2, 1] = Kc[1, 2] = Kc[3, 0] = Kc[0, 3] = (kx - 2.0 * ky) / 6.0    # k32, k41
        Kb = np.zeros((4, 4))
        Fe = np.full(4, f)
        # edges of setBoundaries: (own, other, len, side) with nodes i1..i4 = 0..3
        edges = ((0, 1, w, "bottom"), (1, 2, h, "right"), (2, 3, w, "top"), (0, 3, h, "left"))

        def fac(side, a, b, length):
            if not cyl:
                return 1.0
            if side == "left":
                return x0[i]
            if side == "right":
                return x0[i + 1]
            return r + (-length / 6.0 if node_id.ravel()[nodes[a]] < node_id.ravel()[nodes[b]] else length / 6.0)

        def facmn(side):
            if not cyl:
                return 1.0
            return x0[i] if side == "left" else x0[i + 1] if side == "right" else r

        has, vals = bc["hf"]
        for a, b, length, side in edges:
            if has[nodes[a]] and has[nodes[b]]:
                for p, q in ((a, b), (b, a)):
                    Fe[p] += -0.5e-6 * length * vals[0, nodes[p]] * fac(side, p, q, length)
        has, vals = bc["cv"]
        for a, b, length, side in edges:
            if has[nodes[a]] and has[nodes[b]]:
                c1, c2 = vals[0, nodes[a]], vals[0, nodes[b]]
                for p, q in ((a, b), (b, a)):
                    if cyl:
                        t1, t2 = vals[1, nodes[a]], vals[1, nodes[b]]
                        Fe[p] += 0.125e-6 * length * (c1 + c2) * (t1 + t2) * fac(side, p, q, length)
                    else:
                        Fe[p] += 0.5e-6 * length * vals[0, nodes[p]] * vals[1, nodes[p]]
                    Kb[p, p] += kscale * (c1 + c2) * length / 6.0 * fac(side, p, q, length)
                v = kscale * (c1 + c2) * length / 12.0 * facmn(side)
                Kb[a, b] += v
                Kb[b, a] += v
        has, vals = bc["rd"]
        for a, b, length, side in edges:
            if has[nodes[a]] and has[nodes[b]]:
                for p, q in ((a, b), (b, a)):
                    amb = vals[1, nodes[p]] ** 2
                    t2 = Tf[nodes[p]] ** 2
                    Fe[p] += -0.5e-6 * length * vals[0, nodes[p]] * SB * (t2 * t2 - amb * amb) * fac(side, p, q, length)
        # the cylindrical element adds r (k11 + edge terms), therm2d.cpp:410-420
        wc = r if cyl else 1.0
        K = wc * Kc + (wc if prob.bc_compat else 1.0) * Kb
        ids = [int(node_id.ravel()[nd]) for nd in nodes]
        for a in range(4):
            for b in range(4):
                rows.append(ids[a])
                cols.append(ids[b])
                data.append(K[a, b])
            Fv[ids[a]] += Fe[a]
    A = sp.csr_matrix((np.array(data), (np.array(rows), np.array(cols))), shape=(n_act, n_act))
    return A, Fv


def dirichlet_values(prob, node_id, n_act):
    return F3.dirichlet_values(prob, node_id, n_act)


def to_full(prob, node_id, x, fill=np.nan):
    out = np.full(prob.shape, fill)
    ids = node_id.ravel()
    out.ravel()[ids >= 0] = np.asarray(x)[ids[ids >= 0]]
    return out


def outer_step(prob, T, thickness, numbering, method="direct"):
    node_id, n_act = numbering
    A, Fv = assemble(prob, T, thickness, numbering)
    is_d, vf, vl = dirichlet_values(prob, node_id, n_act)
    A2, b = F3.apply_dirichlet(A, Fv, is_d, vf, vl)
    x = F3.solve(A2, b, method)
    Tn = to_full(prob, node_id, x)
    inactive = node_id < 0
    Tn[inactive] = np.asarray(T)[inactive]
    return Tn, (A2, b, x)


def compute(prob, loops=0, T=None, method="direct"):
    """ThermalFem2DSolver::compute (therm2d.cpp:444-502): (T (n1, n0), toterr, records)."""
    numbering = masked_numbering(prob)
    thickness = element_thickness(prob)
    if T is None:
        T = np.full(prob.shape, float(prob.inittemp))
    active = numbering[0] >= 0
    toterr, loop, records = 0.0, 0, []
    while True:
        T0 = T.copy()
        T, _ = outer_step(prob, T, thickness, numbering, method)
        err = float(np.max(np.abs(T[active] - T0[active]))) if active.any() else 0.0
        maxT = float(max(np.max(T[active]), 0.0)) if active.any() else 0.0
        toterr = max(toterr, err)
        loop += 1
        records.append(F3.LoopRecord(loop, maxT, err))
        if not (err > prob.maxerr and (loops == 0 or loop < loops)):
            break
    return T, toterr, records


def heat_fluxes(prob, T, leaf_height=None):
    """Per-element heat flux [W/m^2], (ne1, ne0, 2) (therm2d.cpp:505-541); excluded elements NaN."""
    n1, n0 = prob.shape
    x0, x1 = (np.asarray(a, np.float64) for a in prob.axes)
    c = _corners(prob.shape)
    t = np.asarray(T, np.float64).ravel()[c]
    ll, lr, ul, ur = t
    temp = 0.25 * (ll + lr + ul + ur)
    if leaf_height is None:
        leaf_height = element_thickness(prob)
    kx, ky = prob.materials.thermk(prob.mat.ravel(), temp, np.asarray(leaf_height).ravel())
    jj, ii = (a.ravel() for a in np.meshgrid(np.arange(n1 - 1), np.arange(n0 - 1), indexing="ij"))
    qx = -0.5e6 * kx * (-ll + lr - ul + ur) / (x0[ii + 1] - x0[ii])
    qy = -0.5e6 * ky * (-ll - lr + ul + ur) / (x1[jj + 1] - x1[jj])
    q = np.stack([qx, qy], axis=-1).reshape((n1 - 1, n0 - 1, 2))
    q[~element_active(prob)] = np.nan
    return q


def conductivity(prob, T, thickness=None):
    """(k_0, k_1) per element at the element-mean temperature (therm2d.cpp:574-597)."""
    c = _corners(prob.shape)
    t = np.asarray(T, np.float64).ravel()[c]
    temp = 0.25 * t.sum(axis=0)
    if thickness is None:
        thickness = element_thickness(prob)
    kx, ky = prob.materials.thermk(prob.mat.ravel(), temp, np.asarray(thickness).ravel())
    out = np.stack([kx, ky], axis=-1).reshape(prob.mat.shape + (2,))
    out[~element_active(prob)] = np.nan
    return out
