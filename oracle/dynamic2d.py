"""CPU oracle of the Dynamic2D / DynamicCyl thermal solvers -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of PLaSK's ``thermal.dynamic.Dynamic2D`` and ``DynamicCyl``
(solvers/thermal/dynamic/femT2d.cpp), on the assembly of oracle/fem2d.py:

* ``set_matrix``  setMatrix: A = theta K + C, B = -(1 - theta) K + C, load F, Dirichlet
                   elimination on A and F                          femT2d.cpp:128-384
* ``compute``     the time loop: X = B T + F, A T = X               femT2d.cpp:387-445

C is the heat capacity with c = cp dens 0.25e-3 w h / timestep per element corner
(femT2d.cpp:167, times the midpoint radius in the cylindrical form, :298): lumped onto the
diagonal (the default) or the consistent bilinear matrix c (4, 2, 1) / 9 by corner
distance (:183-233, 314-362).  As in oracle/dynamic3d.py the Dirichlet nodes hold their values at
every step (the scheme setMatrix prepares; the reference's step loop adds (B T)[r] to
those rows and passes the vectors through aliasing buffers).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import fem2d as F2
from . import fem3d as F3


def _mass(prob, cp, dens, timestep, lumping, numbering):
    node_id, n = numbering
    act = F2.element_active(prob).ravel()
    corners = F2._corners(prob.shape)[:, act]  # LL, LR, UL, UR
    ids = node_id.ravel()[corners]
    x0, x1 = (np.asarray(a, np.float64) for a in prob.axes)
    n1, n0 = prob.shape
    jj, ii = (a.ravel()[act] for a in np.meshgrid(np.arange(n1 - 1), np.arange(n0 - 1), indexing="ij"))
    w, h = x0[ii + 1] - x0[ii], x1[jj + 1] - x1[jj]
    m = prob.mat.ravel()[act]
    c = cp[m] * dens[m] * 0.25 * 1e-12 * h * w / timestep / 1e-9
    if prob.geometry == "cylindrical":
        r = 0.5 * (x0[ii] + x0[ii + 1])
        c = cp[m] * dens[m] * 0.25 * 1e-12 * r * h * w / timestep / 1e-9
    if lumping:
        d = np.zeros(n)
        for a in range(4):
            np.add.at(d, ids[a], c)
        return sp.diags(d).tocsr()
    # corner index a = ci + 2 cj: same corner 4/9, edge neighbours (a ^ b = 1 or 2) 2/9, opposite 1/9
    wgt = {0: 4.0 / 9.0, 1: 2.0 / 9.0, 2: 2.0 / 9.0, 3: 1.0 / 9.0}
    rows, cols, data = [], [], []
    for a in range(4):
        for b in range(4):
            rows.append(ids[a])
            cols.append(ids[b])
            data.append(wgt[a ^ b] * c)
    return sp.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def set_matrix(prob, T, cp, dens, timestep, theta, lumping, numbering, thickness):
    """(A with Dirichlet rows eliminated, B, F with the elimination terms, is_d, v_last)."""
    node_id, n = numbering
    K, Fh = F2.assemble(prob, T, thickness, numbering)
    C = _mass(prob, cp, dens, timestep, lumping, numbering)
    A = (theta * K + C).tocsr()
    B = (-(1.0 - theta) * K + C).tocsr()
    is_d, vf, vl = F2.dirichlet_values(prob, node_id, n)
    A2, Fel = F3.apply_dirichlet(A, Fh, is_d, vf, vl)
    return A2, B, Fel, is_d, vl


def compute(prob, time, cp, dens, T=None, timestep=0.1, theta=0.5, lumping=True, rebuildfreq=0, method="direct"):
    """DynamicThermalFem2DSolver::compute(time): (T in the masked numbering, elapsed time, steps).

    ``T`` starts from inittemp by default; the loop runs while t < time + timestep / 2
    (femT2d.cpp:418-441)."""
    numbering = F2.masked_numbering(prob)
    node_id, n = numbering
    thickness = F2.element_thickness(prob)
    cp = np.asarray(cp, np.float64)
    dens = np.asarray(dens, np.float64)
    if T is None:
        T = np.full(n, float(prob.inittemp))
    full = lambda x: F2.to_full(prob, node_id, x, fill=np.nan)
    A, B, Fel, is_d, vl = set_matrix(prob, full(T), cp, dens, timestep, theta, lumping, numbering, thickness)
    r = rebuildfreq
    time = time + timestep / 2.0
    t = 0.0
    elaps = 0.0
    steps = 0
    while t < time:
        if rebuildfreq and r == 0:
            A, B, Fel, is_d, vl = set_matrix(prob, full(T), cp, dens, timestep, theta, lumping, numbering, thickness)
            r = rebuildfreq
        X = B @ T + Fel
        X[is_d] = vl[is_d]
        T = F3.solve(A, X, method)
        r -= 1
        elaps += timestep
        t += timestep
        steps += 1
    elaps -= timestep
    return T, elaps, steps
