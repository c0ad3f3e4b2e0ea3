"""CPU oracle of the Dynamic3D thermal solver -- TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of PLaSK's ``thermal.dynamic.Dynamic3D``
(solvers/thermal/dynamic/femT3d.cpp), sharing the mesh numbering, conductivity
model, thickness and Dirichlet elimination of oracle/fem3d.py:

* ``set_matrix``  setMatrix: A = theta K + C, B = -(1 - theta) K + C, load F,
                   Dirichlet elimination on A and F               femT3d.cpp:128-252
* ``compute``     the time loop: X = B T + F, A T = X              femT3d.cpp:255-315

C is the heat-capacity matrix with c = cp dens 0.125e-9 dx dy dz / timestep per
element corner (femT3d.cpp:183): lumped onto the diagonal (the default) or the
consistent trilinear mass (8, 4, 2, 1)/27 c (femT3d.cpp:203-226).

Dirichlet nodes hold their value at every step: X[r] = value, A's identity row
returning it.  This is the scheme the reference's setMatrix sets up; its step loop
(femT3d.cpp:291-300) passes the right-hand side and the solution through
reference-counted buffers that alias after the first step (`DataVector<double> T(X)`
shares X's storage, and the Cholesky and NSPCG back ends swap their arguments
differently), and it adds (B T)[r] to the Dirichlet rows because B is never given the
boundary conditions, which on meshes with large substrate elements (c_r > 1) grows
without bound.  The oracle follows the intended theta method instead.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import fem3d as F


def _mass(prob, cp, dens, timestep, lumping, numbering):
    node_id, n = numbering
    act = F.element_active(prob).ravel()
    shape = prob.shape
    nodes_c = F._element_nodes(shape)[:, act]
    ids = node_id.ravel()[nodes_c]
    x0, x1, x2 = (np.asarray(a, np.float64) for a in prob.axes)
    ne = tuple(s - 1 for s in shape)
    kk, jj, ii = (a.ravel()[act] for a in np.meshgrid(*(np.arange(m) for m in ne), indexing="ij"))
    dx, dy, dz = x0[ii + 1] - x0[ii], x1[jj + 1] - x1[jj], x2[kk + 1] - x2[kk]
    m = prob.mat.ravel()[act]
    c = cp[m] * dens[m] * 0.125e-9 * dx * dy * dz / timestep
    if lumping:
        d = np.zeros(n)
        for a in range(8):
            np.add.at(d, ids[a], c)
        return sp.diags(d).tocsr()
    w = {0: 8.0 / 27.0, 1: 4.0 / 27.0, 2: 4.0 / 27.0, 4: 4.0 / 27.0, 3: 2.0 / 27.0, 5: 2.0 / 27.0, 6: 2.0 / 27.0,
         7: 1.0 / 27.0}
    rows, cols, data = [], [], []
    for a in range(8):
        for b in range(8):
            rows.append(ids[a]); cols.append(ids[b]); data.append(w[a ^ b] * c)
    return sp.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def set_matrix(prob, T, cp, dens, timestep, theta, lumping, numbering, thickness):
    """(A with Dirichlet rows eliminated, B, F with the elimination terms)."""
    node_id, n = numbering
    K, Fh, _, _ = F.assemble(prob, T, thickness, node_id, n)
    C = _mass(prob, cp, dens, timestep, lumping, numbering)
    A = (theta * K + C).tocsr()
    B = (-(1.0 - theta) * K + C).tocsr()
    is_d, vf, vl = F.dirichlet_values(prob, node_id, n)
    A2, Fel = F.apply_dirichlet(A, Fh, is_d, vf, vl)
    return A2, B, Fel, is_d, vl


def compute(prob, time, cp, dens, T=None, timestep=0.1, theta=0.5, lumping=True, rebuildfreq=0, method="direct"):
    """DynamicThermalFem3DSolver::compute(time): returns (T_full, elapsed time, steps).

    ``T`` is the nodal temperature in the masked numbering to start from (inittemp by
    default); the loop runs while t < time + timestep / 2 (femT3d.cpp:283-307)."""
    numbering = F.masked_numbering(prob)
    node_id, n = numbering
    thickness = F.element_thickness(prob)
    cp = np.asarray(cp, np.float64)
    dens = np.asarray(dens, np.float64)
    if T is None:
        T = np.full(n, float(prob.inittemp))
    full = lambda x: F.to_full(prob, node_id, x, fill=np.nan)
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
        T = F.solve(A, X, method)
        r -= 1
        elaps += timestep
        t += timestep
        steps += 1
    elaps -= timestep
    return T, elaps, steps
