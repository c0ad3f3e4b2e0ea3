"""CPU oracle for the 3D FEM thermal hot path (Static3D) -- TEST INFRASTRUCTURE ONLY.

This module is the checker for the GPU solver: only tests, the smoke check and
the CPU-baseline leg of the benchmark may import it.  The product path never
calls it.

It restates, in FP64 numpy, what PLaSK's ``thermal.static.Static3D`` does for
one ``compute()`` call.  Every function cites the reference lines it follows
(paths relative to the PLaSK source tree):

* ``element_thickness``      solvers/thermal/static/therm3d.cpp:81-113
* ``masked_numbering``       plask/mesh/rectangular_masked3d.cpp:40-64,
                             plask/common/fem/fem_solver.hpp:182-189
* ``reference_order``        plask/mesh/rectilinear3d.cpp:20-33, 74-85
* ``first_match``            plask/mesh/boundary_conditions.hpp:182-186
* ``assemble``               solvers/thermal/static/therm3d.cpp:141-279
                             (including the 3D boundary-face placement quirk:
                             face terms land on element corners 0..3 and the
                             radiation term reads the temperatures of global
                             nodes 0..7)
* ``apply_dirichlet``        plask/common/fem/matrix.hpp:111-145
* ``solve_band_cholesky``    plask/common/fem/cholesky_matrix.hpp:58-119
                             (LAPACK dpbtrf/dpbtrs, UPLO='L')
* ``compute``                solvers/thermal/static/therm3d.cpp:281-340
* ``heat_fluxes``            solvers/thermal/static/therm3d.cpp:342-384

Array conventions: node arrays have shape ``(n2, n1, n0)`` (axis 0 fastest),
element arrays ``(n2-1, n1-1, n0-1)``; axis 2 is the vertical axis.  Lengths
are in micrometres, heat densities in W/m^3, conductivities in W/(m K).

Parity of the assembly is pinned by analytic known-answer tests (1D layered
slab, linear patch field) and by the Shockley3D analytic-current test of the
reference; the linear solve is pinned against NSPCG compiled from the
reference's own ``extlib/nspcg/nspcg.c`` where that build is available.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.linalg.lapack as lapack
import scipy.sparse as sp
import scipy.sparse.linalg as spla

SB = 5.670373e-8  # plask/phys/constants.hpp:41

# corner c -> (ci, cj, ck) bits, therm3d.cpp:190-197 (0=LoLoLo, 1=UpLoLo, 2=LoUpLo, ... 7=UpUpUp)
CORNERS = np.array([[c & 1, (c >> 1) & 1, (c >> 2) & 1] for c in range(8)], dtype=np.int64)
# element faces as corner quadruples, therm3d.cpp:150
WALLS = ((0, 1, 2, 3), (4, 5, 6, 7), (0, 2, 4, 6), (1, 3, 5, 7), (0, 1, 4, 5), (2, 3, 6, 7))


@dataclasses.dataclass
class Materials:
    """Per-material thermal conductivity model k(T) = k300 * (300/T)**p * h**hexp.

    ``kz_ratio`` gives the vertical/lateral anisotropy (k_z = kz_ratio * k_xy),
    ``hexp`` the optional dependence on the layer thickness h that PLaSK passes
    as the second argument of ``Material::thermk(T, h)``; ``empty`` marks
    materials of kind EMPTY (dropped by the masked mesh).
    """

    k300: np.ndarray
    p: np.ndarray
    kz_ratio: np.ndarray | None = None
    hexp: np.ndarray | None = None
    empty: np.ndarray | None = None
    # tabulated k(T): {material id: (T, k_xy, k_z or None)}, replacing the power law of that
    # material (piecewise linear in T, constant beyond the ends; h**hexp still applies)
    tables: dict | None = None

    def __post_init__(self):
        self.k300 = np.asarray(self.k300, dtype=np.float64)
        n = self.k300.size
        self.p = np.asarray(self.p, dtype=np.float64)
        self.kz_ratio = np.ones(n) if self.kz_ratio is None else np.asarray(self.kz_ratio, dtype=np.float64)
        self.hexp = np.zeros(n) if self.hexp is None else np.asarray(self.hexp, dtype=np.float64)
        self.empty = np.zeros(n, bool) if self.empty is None else np.asarray(self.empty, dtype=bool)

    def thermk(self, m, T, h):
        """(k_xy, k_z) of material ids ``m`` at temperature ``T`` and thickness ``h``."""
        m = np.asarray(m)
        kxy = self.k300[m] * (300.0 / T) ** self.p[m]
        he = self.hexp[m]
        if np.any(he != 0):
            kxy = kxy * np.where(he != 0, h ** he, 1.0)
        kz = kxy * self.kz_ratio[m]
        if self.tables:
            Tb = np.broadcast_to(np.asarray(T, np.float64), m.shape)
            hb = np.broadcast_to(np.asarray(h, np.float64), m.shape) if h is not None else None
            kxy, kz = np.array(kxy, np.float64, copy=True), np.array(kz, np.float64, copy=True)
            for mid, tab in self.tables.items():
                sel = m == mid
                if not np.any(sel):
                    continue
                a, c = table_k(tab, Tb[sel])
                if self.hexp[mid] != 0:
                    f = hb[sel] ** self.hexp[mid]
                    a, c = a * f, c * f
                kxy[sel], kz[sel] = a, c
        return kxy, kz


def table_k(tab, T):
    """(k_xy, k_z) of a tabulated material at temperatures T: linear between the points,
    constant beyond the first and the last (the GPU's mat_thermk evaluates the same)."""
    t = np.asarray(tab[0], np.float64)
    a = np.asarray(tab[1], np.float64)
    c = a if len(tab) < 3 or tab[2] is None else np.asarray(tab[2], np.float64)
    T = np.asarray(T, np.float64)
    hi = np.clip(np.searchsorted(t, T, side="right"), 1, max(len(t) - 1, 1))
    lo = hi - 1
    if len(t) == 1:
        return np.full(T.shape, a[0]), np.full(T.shape, c[0])
    w = (T - t[lo]) / (t[hi] - t[lo])
    ka = a[lo] + w * (a[hi] - a[lo])
    kc = c[lo] + w * (c[hi] - c[lo])
    below, above = ~(T > t[0]), T >= t[-1]
    ka = np.where(below, a[0], np.where(above, a[-1], ka))
    kc = np.where(below, c[0], np.where(above, c[-1], kc))
    return ka, kc


@dataclasses.dataclass
class Problem:
    """One Static3D problem: mesh axes, element materials, heat, and boundary conditions.

    Boundary-condition lists keep PLaSK's order (first matching condition wins
    for heat flux, convection and radiation; temperature conditions are applied
    in list order).  Each place is a boolean node mask of shape (n2, n1, n0).

    * ``temperature``: [(mask, T)]
    * ``heatflux``:    [(mask, q)]            q in W/m^2
    * ``convection``:  [(mask, h, T_amb)]     h in W/(m^2 K)
    * ``radiation``:   [(mask, eps, T_amb)]
    """

    axes: tuple
    mat: np.ndarray
    materials: Materials
    heat: np.ndarray
    temperature: list = dataclasses.field(default_factory=list)
    heatflux: list = dataclasses.field(default_factory=list)
    convection: list = dataclasses.field(default_factory=list)
    radiation: list = dataclasses.field(default_factory=list)
    order: str = "012"
    inittemp: float = 300.0
    maxerr: float = 0.05
    empty_elements: str = "exclude"  # "exclude" (masked mesh) or "include"
    leaf_height: np.ndarray | None = None  # per element, for heat_fluxes (default: thickness)

    @property
    def shape(self):
        return tuple(len(a) for a in self.axes[::-1])  # (n2, n1, n0)


# ----------------------------------------------------------------------------------------
# mesh numbering


def reference_order(shape, order: str):
    """Index of every node in the reference iteration order.

    ``order`` is PLaSK's ``ORDER_<major><medium><minor>`` string, e.g. "012" means
    axis 2 changes fastest (rectilinear3d.cpp:20-33).  Returns an int64 array
    of shape ``shape`` = (n2, n1, n0).
    """
    n2, n1, n0 = shape
    n = (n0, n1, n2)
    a, b, c = (int(ch) for ch in order)
    i0, i1, i2 = np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij")
    idx = {0: i0, 1: i1, 2: i2}
    ref = idx[c] + n[c] * (idx[b] + n[b] * idx[a])
    return np.ascontiguousarray(ref.transpose(2, 1, 0)).astype(np.int64)


def optimal_order(n0, n1, n2):
    """RectilinearMesh3D::setOptimalIterationOrder (rectilinear3d.cpp:74-85)."""
    n = (n0, n1, n2)
    for f, s, t in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        if n[t] <= n[s] <= n[f]:
            return f"{f}{s}{t}"
    return "210"


def element_active(prob: Problem):
    """Elements kept by the masked mesh (fem_solver.hpp:182-189)."""
    if prob.empty_elements == "include":
        return np.ones(prob.mat.shape, bool)
    return ~prob.materials.empty[prob.mat]


def masked_numbering(prob: Problem):
    """Masked-mesh node numbering (rectangular_masked3d.cpp:40-64).

    Nodes touched by at least one active element keep the full-mesh iteration
    order and are numbered consecutively.  Returns (node_id, n_active) where
    node_id has shape (n2, n1, n0) and is -1 for dropped nodes.
    """
    act = element_active(prob)
    n2, n1, n0 = prob.shape
    used = np.zeros((n2, n1, n0), bool)
    for ck in (0, 1):
        for cj in (0, 1):
            for ci in (0, 1):
                used[ck:n2 - 1 + ck, cj:n1 - 1 + cj, ci:n0 - 1 + ci] |= act
    ref = reference_order(prob.shape, prob.order)
    order = np.argsort(ref[used], kind="stable")
    node_id = np.full((n2, n1, n0), -1, np.int64)
    flat = np.flatnonzero(used.ravel())
    ids = np.empty(flat.size, np.int64)
    ids[order] = np.arange(flat.size)
    node_id.ravel()[flat] = ids
    return node_id, int(flat.size)


def element_thickness(prob: Problem):
    """Height of the vertical run of equal-material elements (therm3d.cpp:81-113)."""
    mat = prob.mat
    z = np.asarray(prob.axes[2], np.float64)
    ne2 = mat.shape[0]
    kidx = np.arange(ne2)[:, None, None] * np.ones(mat.shape[1:], np.int64)[None]
    # a run starts at k when k == 0 or the material differs from the element below
    starts = np.ones(mat.shape, bool)
    starts[1:] = mat[1:] != mat[:-1]
    start = np.maximum.accumulate(np.where(starts, kidx, 0), axis=0)
    # a run ends after k when k is the last element or the material differs from the one above
    ends = np.ones(mat.shape, bool)
    ends[:-1] = mat[1:] != mat[:-1]
    stop = np.minimum.accumulate(np.where(ends, kidx + 1, ne2)[::-1], axis=0)[::-1]
    return z[stop] - z[start]


# ----------------------------------------------------------------------------------------
# assembly


def _element_nodes(shape):
    """(8, ne) canonical node indices of element corners in therm3d.cpp:190-197 order."""
    n2, n1, n0 = shape
    k, j, i = np.meshgrid(np.arange(n2 - 1), np.arange(n1 - 1), np.arange(n0 - 1), indexing="ij")
    base = (i + n0 * (j + n1 * k)).ravel()
    off = CORNERS[:, 0] + n0 * (CORNERS[:, 1] + n1 * CORNERS[:, 2])
    return base[None, :] + off[:, None]


def first_match(prob_list, shape, nvals):
    """Per node: values of the first condition whose place contains it (boundary_conditions.hpp:182-186).

    Returns (has, vals) with vals of shape (nvals, N).
    """
    N = int(np.prod(shape))
    has = np.zeros(N, bool)
    vals = np.zeros((nvals, N))
    for cond in prob_list:
        m = np.asarray(cond[0], bool).ravel() & ~has
        for v in range(nvals):
            vals[v, m] = cond[1 + v]
        has |= m
    return has, vals


def element_k(prob: Problem, T, thickness=None):
    """Per-element (k_xy, k_z) at the 8-node average temperature (therm3d.cpp:208-213)."""
    shape = prob.shape
    nodes = _element_nodes(shape)
    Tf = np.asarray(T, np.float64).ravel()
    temp = Tf[nodes].sum(axis=0) * 0.125
    if thickness is None:
        thickness = element_thickness(prob)
    return prob.materials.thermk(prob.mat.ravel(), temp, thickness.ravel())


def assemble(prob: Problem, T, thickness=None, node_id=None, n_active=None):
    """Stiffness matrix and load vector before Dirichlet elimination (therm3d.cpp:170-276).

    ``T`` is the current nodal temperature on the full grid (n2, n1, n0).
    Returns (A, F, node_id, n_active) where A is a symmetric scipy CSR matrix over the
    masked-mesh numbering and F the load vector.
    """
    ids, K, F, node_id, n_active = element_terms(prob, T, thickness, node_id, n_active)
    rows, cols, data = [], [], []
    for (a, b), v in K.items():
        ra, cb = ids[a], ids[b]
        rows.append(ra); cols.append(cb); data.append(v)
        if a != b:
            rows.append(cb); cols.append(ra); data.append(v)
    A = sp.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n_active, n_active))
    Fv = np.zeros(n_active)
    for a in range(8):
        np.add.at(Fv, ids[a], F[a])
    return A, Fv, node_id, n_active


def element_terms(prob: Problem, T, thickness=None, node_id=None, n_active=None):
    """Per-element stiffness entries and loads of setMatrix (therm3d.cpp:186-268).

    Returns (ids, K, F, node_id, n_active): ids (8, ne) masked node ids of the
    active elements' corners, K {(a, b): values} for b <= a (lower triangle of
    K_e including the boundary-face terms) and F [8 arrays] the element loads.
    """
    shape = prob.shape
    n2, n1, n0 = shape
    if node_id is None:
        node_id, n_active = masked_numbering(prob)
    act = element_active(prob).ravel()
    nodes_c = _element_nodes(shape)[:, act]  # canonical
    ids = node_id.ravel()[nodes_c]  # masked ids
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    ne = (n2 - 1, n1 - 1, n0 - 1)
    kk, jj, ii = (a.ravel()[act] for a in np.meshgrid(*(np.arange(m) for m in ne), indexing="ij"))
    dx = x0[ii + 1] - x0[ii]
    dy = x1[jj + 1] - x1[jj]
    dz = x2[kk + 1] - x2[kk]
    Tf = np.asarray(T, np.float64).ravel()
    temp = Tf[nodes_c].sum(axis=0) * 0.125
    if thickness is None:
        thickness = element_thickness(prob)
    ky, kz = prob.materials.thermk(prob.mat.ravel()[act], temp, thickness.ravel()[act])
    ky = ky * 1e-6
    kz = kz * 1e-6
    kx = ky.copy()
    kx = kx / dx; kx = kx * dy; kx = kx * dz  # therm3d.cpp:218-220, same operation order
    ky = ky * dx; ky = ky / dy; ky = ky * dz
    kz = kz * dx; kz = kz * dy; kz = kz / dz
    f = 0.125e-18 * dx * dy * dz * prob.heat.ravel()[act]

    # K[a][b] depends only on a^b (therm3d.cpp:227-237)
    g = {
        0: (kx + ky + kz) / 9.0,
        1: (-2.0 * kx + ky + kz) / 18.0,
        2: (kx - 2.0 * ky + kz) / 18.0,
        4: (kx + ky - 2.0 * kz) / 18.0,
        6: (kx - 2.0 * ky - 2.0 * kz) / 36.0,
        5: (-2.0 * kx + ky - 2.0 * kz) / 36.0,
        3: (-2.0 * kx - 2.0 * ky + kz) / 36.0,
        7: -(kx + ky + kz) / 36.0,
    }
    K = {}
    for a in range(8):
        for b in range(a + 1):
            K[(a, b)] = g[a ^ b].copy()
    F = [f.copy() for _ in range(8)]

    # boundary faces (therm3d.cpp:141-168, 243-268), with the reference's placement
    N = n0 * n1 * n2
    areas = (dx * dy, dy * dz, dz * dx)
    ref_ids = node_id.ravel()  # masked id == position in reference iteration order
    inv = np.full(n_active, -1, np.int64)
    inv[ref_ids[ref_ids >= 0]] = np.flatnonzero(ref_ids >= 0)
    # temperatures of global (masked) nodes 0..7, read by the radiation term (therm3d.cpp:265)
    Tglob = Tf[inv[: min(8, n_active)]]

    def faces(has, vals, Ffun, Kfun):
        hv = has[nodes_c]
        for side, wall in enumerate(WALLS):
            sel = hv[wall[0]] & hv[wall[1]] & hv[wall[2]] & hv[wall[3]]
            if not np.any(sel):
                continue
            area = areas[side // 2][sel]
            for i in range(4):
                vi = vals[:, nodes_c[wall[i], sel]]
                if Ffun is not None:
                    F[i][sel] += Ffun(area, vi, wall[i])
                if Kfun is None:
                    continue
                for j in range(i + 1):
                    vj = vals[:, nodes_c[wall[j], sel]]
                    ij = i ^ j
                    edge = ij in (1, 2, 4)
                    K[(i, j)][sel] += Kfun(area, vi, vj, i == j, edge)

    has, vals = first_match(prob.heatflux, shape, 1)
    if prob.heatflux:
        faces(has, vals, lambda area, v, w: -0.25e-12 * area * v[0], None)
    has, vals = first_match(prob.convection, shape, 2)
    if prob.convection:
        faces(has, vals, lambda area, v, w: 0.25e-12 * area * v[0] * v[1],
              lambda area, v1, v2, same, edge: 0.125e-12 * area * (v1[0] + v2[0]) / (9.0 if same else 18.0 if edge else 36.0))
    has, vals = first_match(prob.radiation, shape, 2)
    if prob.radiation:
        def rad(area, v, w):
            a = v[1] * v[1]
            t = Tglob[w] * Tglob[w]
            return -0.25e-12 * area * v[0] * SB * (t * t - a * a)
        faces(has, vals, rad, None)

    return ids, K, F, node_id, n_active


def dirichlet_values(prob: Problem, node_id, n_active):
    """Dirichlet rows in the order BandMatrix::setBC sees them (matrix.hpp:111-145).

    Returns (is_d, v_first, v_last): v_first is the value of the first condition
    listing the node (it is the one eliminated from neighbouring rows), v_last
    the value of the last one (it ends up in the right-hand side).
    """
    is_d = np.zeros(n_active, bool)
    v_first = np.zeros(n_active)
    v_last = np.zeros(n_active)
    ids = node_id.ravel()
    for mask, val in prob.temperature:
        m = np.asarray(mask, bool).ravel() & (ids >= 0)
        r = ids[m]
        new = r[~is_d[r]]
        v_first[new] = val
        is_d[r] = True
        v_last[r] = val
    return is_d, v_first, v_last


def apply_dirichlet(A, F, is_d, v_first, v_last):
    """Symmetric elimination of Dirichlet rows (matrix.hpp:132-145)."""
    A = A.tocsr()
    b = F - A[:, is_d] @ v_first[is_d]
    b[is_d] = v_last[is_d]
    keep = ~is_d
    Dk = sp.diags(keep.astype(np.float64))
    A2 = (Dk @ A @ Dk + sp.diags(is_d.astype(np.float64))).tocsr()
    return A2, b


# ----------------------------------------------------------------------------------------
# linear solves


def solve_band_cholesky(A, b, perm=None):
    """LAPACK dpbtrf/dpbtrs with UPLO='L' on the band of A (cholesky_matrix.hpp:90-111).

    ``perm`` is ignored: A is already in the reference (masked-mesh) numbering,
    whose bandwidth is what the reference factorises.
    """
    A = A.tocoo()
    lower = A.row >= A.col
    r, c, v = A.row[lower], A.col[lower], A.data[lower]
    kd = int((r - c).max()) if r.size else 0
    n = A.shape[0]
    ab = np.zeros((kd + 1, n), order="F")
    np.add.at(ab, (r - c, c), v)
    cfac, info = lapack.dpbtrf(ab, lower=1)
    if info > 0:
        raise ArithmeticError(f"leading minor of order {info} of the stiffness matrix is not positive-definite")
    if info < 0:
        raise ValueError(f"argument {-info} of dpbtrf has an illegal value")
    x, info = lapack.dpbtrs(cfac, b, lower=1)
    if info != 0:
        raise ValueError(f"dpbtrs failed: info={info}")
    return x


def solve_direct(A, b):
    """Sparse LU solve (SuperLU); same exact solution as the band Cholesky, faster at size."""
    return spla.spsolve(A.tocsc(), b)


def solve(A, b, method="cholesky"):
    if method == "cholesky":
        return solve_band_cholesky(A, b)
    if method == "direct":
        return solve_direct(A, b)
    raise ValueError(method)


# ----------------------------------------------------------------------------------------
# the outer loop


@dataclasses.dataclass
class LoopRecord:
    loop: int
    maxT: float
    err: float


def to_full(prob, node_id, x, fill=np.nan):
    out = np.full(prob.shape, fill)
    ids = node_id.ravel()
    out.ravel()[ids >= 0] = x[ids[ids >= 0]]
    return out


def from_full(node_id, n_active, T):
    ids = node_id.ravel()
    x = np.empty(n_active)
    x[ids[ids >= 0]] = np.asarray(T).ravel()[ids >= 0]
    return x


def outer_step(prob, T, method="cholesky", thickness=None, numbering=None):
    """One pass of the Picard loop body: assemble with T, eliminate, solve (therm3d.cpp:311-315)."""
    node_id, n_active = numbering if numbering is not None else masked_numbering(prob)
    A, F, _, _ = assemble(prob, T, thickness, node_id, n_active)
    is_d, vf, vl = dirichlet_values(prob, node_id, n_active)
    A2, b = apply_dirichlet(A, F, is_d, vf, vl)
    x = solve(A2, b, method)
    Tn = to_full(prob, node_id, x, fill=np.nan)
    inactive = node_id < 0
    Tn[inactive] = np.asarray(T)[inactive]
    return Tn, (A2, b, x)


def compute(prob: Problem, loops=0, T=None, method="cholesky", log=None):
    """ThermalFem3DSolver::compute (therm3d.cpp:281-340).

    Returns (T, toterr, records): the final nodal temperature (n2, n1, n0), the
    largest per-loop correction, and one LoopRecord per outer iteration.
    """
    numbering = masked_numbering(prob)
    thickness = element_thickness(prob)
    if T is None:
        T = np.full(prob.shape, float(prob.inittemp))
    active = numbering[0] >= 0
    toterr = 0.0
    loop = 0
    records = []
    while True:
        T0 = T.copy()
        T, _ = outer_step(prob, T, method, thickness, numbering)
        err = float(np.max(np.abs(T[active] - T0[active]))) if active.any() else 0.0
        maxT = float(max(np.max(T[active]), 0.0)) if active.any() else 0.0
        toterr = max(toterr, err)
        loop += 1
        records.append(LoopRecord(loop, maxT, err))
        if log is not None:
            log(f"Loop {loop}({loop}): max(T) = {maxT:.3f} K, error = {err:g} K")
        if not (err > prob.maxerr and (loops == 0 or loop < loops)):
            break
    return T, toterr, records


def heat_fluxes(prob: Problem, T, leaf_height=None):
    """Per-element heat flux [W/m^2] (therm3d.cpp:342-384).

    The conductivity is evaluated with the leaf's bounding-box height (not the
    layer-run thickness); ``leaf_height`` defaults to the run thickness, which
    is the same for layered structures built from one block per layer.
    Returns an array (ne2, ne1, ne0, 3); excluded elements are NaN.
    """
    shape = prob.shape
    n2, n1, n0 = shape
    nodes = _element_nodes(shape)
    Tf = np.asarray(T, np.float64).ravel()
    t = Tf[nodes]  # (8, ne)
    temp = 0.125 * (t[0] + t[4] + t[2] + t[6] + t[1] + t[5] + t[3] + t[7])
    if leaf_height is None:
        leaf_height = prob.leaf_height if prob.leaf_height is not None else element_thickness(prob)
    kxy, kz = prob.materials.thermk(prob.mat.ravel(), temp, np.asarray(leaf_height).ravel())
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    ne = (n2 - 1, n1 - 1, n0 - 1)
    kk, jj, ii = (a.ravel() for a in np.meshgrid(*(np.arange(m) for m in ne), indexing="ij"))
    lll, ull, lul, uul, llu, ulu, luu, uuu = t
    qx = -0.25e6 * kxy * (-lll - llu - lul - luu + ull + ulu + uul + uuu) / (x0[ii + 1] - x0[ii])
    qy = -0.25e6 * kxy * (-lll - llu + lul + luu - ull - ulu + uul + uuu) / (x1[jj + 1] - x1[jj])
    qz = -0.25e6 * kz * (-lll + llu - lul + luu - ull + ulu - uul + uuu) / (x2[kk + 1] - x2[kk])
    q = np.stack([qx, qy, qz], axis=-1).reshape(ne + (3,))
    act = element_active(prob)
    q[~act] = np.nan
    return q


def relative_residual(A, b, x):
    r = b - A @ x
    return float(np.linalg.norm(r) / max(np.linalg.norm(b), 1e-300))


def _side(shape, side):
    m = np.zeros(shape, bool)
    sl = {"bottom": (0,), "top": (-1,), "left": (slice(None), 0), "right": (slice(None), -1),
          "back": (slice(None), slice(None), 0), "front": (slice(None), slice(None), -1)}[side]
    m[sl] = True
    return m


def _place(shape, place):
    if isinstance(place, str):
        return _side(shape, place)
    return np.asarray(place, bool).reshape(shape)


def from_structure(s, order=None, empty_elements="exclude"):
    """Build a Problem from a structure description (axes, element material ids,
    material table, heat, boundary conditions on named sides or node masks)."""
    shape = tuple(len(a) for a in s.axes[::-1])
    if order is None:
        order = optimal_order(len(s.axes[0]), len(s.axes[1]), len(s.axes[2]))
    mats = Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty, getattr(s, "ktables", None))
    return Problem(
        axes=tuple(np.asarray(a, np.float64) for a in s.axes), mat=np.asarray(s.mat), materials=mats,
        heat=np.asarray(s.heat, np.float64),
        temperature=[(_place(shape, c[0]), c[1]) for c in s.temperature],
        heatflux=[(_place(shape, c[0]), c[1]) for c in s.heatflux],
        convection=[(_place(shape, c[0]), c[1], c[2]) for c in s.convection],
        radiation=[(_place(shape, c[0]), c[1], c[2]) for c in s.radiation],
        order=order, inittemp=s.inittemp, maxerr=s.maxerr, empty_elements=empty_elements)
