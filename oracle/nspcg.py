"""NSPCG (the reference's ``algorithm="iterative"`` solver) for the oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_ref/libnspcg_ref.so`` (NSPCG compiled from the reference's
own ``extlib/nspcg/nspcg.c`` by ``make -C oracle ref``) and solves the
oracle's assembled systems in the reference's 14-diagonal symmetric storage
(plask/common/fem/iterative_matrix.hpp:373-393):

    offsets {0, 1, m-1, m, m+1, M-m-1, M-m, M-m+1, M-1, M, M+1, M+m-1, M+m, M+m+1}
    m = n_minor, M = n_minor * n_medium,   coef[c + N d] = A(c, c + offset[d])

with the reference defaults: IC preconditioner, CG accelerator, maxit 1000,
zeta 1e-6, a new factorisation every nfact = 10 solves
(iterative_matrix.hpp:50-94, 141-177).
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

from . import fem3d as O

LIB = pathlib.Path(__file__).resolve().parent / "_ref" / "libnspcg_ref.so"
_lib = None


def available():
    return LIB.exists()


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} is not built (make -C oracle ref, needs the reference tree)")
        lib = C.CDLL(str(LIB))
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        lib.oracle_nspcg_cg.restype = C.c_int
        lib.oracle_nspcg_cg.argtypes = [C.c_int, C.c_int, dp, ip, dp, dp, C.c_int, C.c_int, C.c_double, C.c_int,
                                        C.c_int, C.c_int, dp, ip, ip, ip, ip, dp]
        _lib = lib
    return _lib


def band_offsets(prob):
    """The 14 stored diagonals of SparseBandMatrix for the problem's mesh order."""
    a, b, c = (int(ch) for ch in prob.order)
    n = (len(prob.axes[0]), len(prob.axes[1]), len(prob.axes[2]))
    m = n[c]
    M = n[c] * n[b]
    return np.array([0, 1, m - 1, m, m + 1, M - m - 1, M - m, M - m + 1, M - 1, M, M + 1, M + m - 1, M + m, M + m + 1],
                    np.int32), m, M


def diagonal_storage(A, offsets):
    """coef[c + N d] = A(c, c + offsets[d]) for the (eliminated, symmetric) matrix A."""
    A = A.tocsr()
    N = A.shape[0]
    coef = np.zeros((len(offsets), N))
    for d, off in enumerate(offsets):
        c = np.arange(N - off)
        coef[d, : N - off] = np.asarray(A[c, c + off]).ravel()
    return np.ascontiguousarray(coef.ravel())


class NspcgSolver:
    """Stateful NSPCG solve as SparseMatrix keeps it between outer loops (factorisation reuse)."""

    def __init__(self, prob, precond="ic", maxit=1000, zeta=1e-6, nfact=10):
        self.prob = prob
        self.offsets, m, M = band_offsets(prob)
        self.kblsz = m - 1
        self.nbl2d = M - m - 1
        self.precond = 0 if precond == "ic" else 1
        self.maxit, self.zeta, self.nfact = maxit, zeta, nfact
        self.ifact = 1
        self.wksp = None
        self.iwksp = None
        self.iters = 0
        self.final_zeta = 0.0
        self.ier = 0

    def solve(self, A, b, x0):
        lib = _load()
        N = A.shape[0]
        mdim = len(self.offsets)
        coef = diagonal_storage(A, self.offsets)
        jcoef = np.ascontiguousarray(self.offsets, np.int32)
        # iterative_matrix.hpp:149-150: refactorise every nfact calls
        self.ifact -= 1
        ifact = 1 if self.ifact == 0 else 0
        if self.ifact <= 0:
            self.ifact = self.nfact
        nw = 3 * N + 2 * self.maxit + N * mdim + max(self.kblsz, 1)
        inw = mdim + max(2 * N, mdim * mdim + mdim)
        if self.wksp is None or self.wksp.size < nw:
            self.wksp = np.zeros(nw)
            ifact = 1
        if self.iwksp is None or self.iwksp.size < inw:
            self.iwksp = np.zeros(inw, np.int32)
            ifact = 1
        u = np.ascontiguousarray(x0, np.float64).copy()
        rhs = np.ascontiguousarray(b, np.float64).copy()
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        while True:
            nwv, inwv = C.c_int(self.wksp.size), C.c_int(self.iwksp.size)
            it, zt = C.c_int(0), C.c_double(0.0)
            ier = lib.oracle_nspcg_cg(N, mdim, coef.ctypes.data_as(dp), jcoef.ctypes.data_as(ip), u.ctypes.data_as(dp),
                                      rhs.ctypes.data_as(dp), self.precond, self.maxit, self.zeta, ifact, self.kblsz,
                                      self.nbl2d, self.wksp.ctypes.data_as(dp), C.byref(nwv),
                                      self.iwksp.ctypes.data_as(ip), C.byref(inwv), C.byref(it), C.byref(zt))
            if ier == -2 and nwv.value > self.wksp.size:
                self.wksp = np.zeros(nwv.value)
                ifact = 1
                continue
            if ier == -3 and inwv.value > self.iwksp.size:
                self.iwksp = np.zeros(inwv.value, np.int32)
                ifact = 1
                continue
            break
        self.iters, self.final_zeta, self.ier = it.value, zt.value, ier
        if ier < 0:
            raise ArithmeticError(f"NSPCG error {ier}")
        return u


def compute_iterative(prob, loops=0, T=None, **kw):
    """Static3D compute() with algorithm="iterative" (NSPCG), oracle assembly.

    The iterative algorithm includes empty elements by default (fem_solver.hpp:182-189).
    Returns (T, toterr, records, iterations per loop).
    """
    numbering = O.masked_numbering(prob)
    node_id, n_active = numbering
    thickness = O.element_thickness(prob)
    solver = NspcgSolver(prob, **kw)
    if T is None:
        T = np.full(prob.shape, float(prob.inittemp))
    toterr, loop, records, iters = 0.0, 0, [], []
    while True:
        T0 = T.copy()
        A, F, _, _ = O.assemble(prob, T, thickness, node_id, n_active)
        is_d, vf, vl = O.dirichlet_values(prob, node_id, n_active)
        A2, b = O.apply_dirichlet(A, F, is_d, vf, vl)
        x = solver.solve(A2, b, O.from_full(node_id, n_active, T))
        T = O.to_full(prob, node_id, x)
        err = float(np.max(np.abs(T - T0)))
        toterr = max(toterr, err)
        loop += 1
        records.append(O.LoopRecord(loop, float(np.max(T)), err))
        iters.append(solver.iters)
        converged = solver.ier != 1
        if not ((not converged or err > prob.maxerr) and (loops == 0 or loop < loops)):
            break
    return T, toterr, records, iters
