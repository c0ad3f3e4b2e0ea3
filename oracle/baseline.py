"""CPU baseline of the reference's default Static3D path -- TEST INFRASTRUCTURE ONLY.

The reference's Static3D defaults to ``algorithm="iterative"`` (therm3d.cpp:32):
setMatrix assembles the 14-diagonal symmetric SparseBandMatrix
(plask/common/fem/iterative_matrix.hpp:373-418), Dirichlet rows are eliminated
by SparseBandMatrix::setBC (iterative_matrix.hpp:462-485), and NSPCG solves
with the IC preconditioner and CG (iterative_matrix.hpp:141-339).

Here the assembly is the oracle's numpy restatement written straight into
that diagonal storage, and the solve is either NSPCG compiled from the
reference tree (``oracle/_ref``) or the oracle's IC(0)-PCG restatement in C
(``oracle/_build/liboracle_iccg.so``), both single-threaded like NSPCG.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess
import time

import numpy as np

from . import fem3d as O
from . import nspcg as NS

HERE = pathlib.Path(__file__).resolve().parent
ICCG = HERE / "_build" / "liboracle_iccg.so"


def _iccg_lib():
    if not ICCG.exists():
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    lib = C.CDLL(str(ICCG))
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.oracle_iccg.restype = C.c_int
    lib.oracle_iccg.argtypes = [C.c_long, C.c_int, ip, dp, dp, C.c_int, dp, dp, C.c_int, C.c_double, ip, dp]
    return lib


def assemble_diagonal(prob, T, thickness=None, numbering=None):
    """setMatrix + applyBC into the reference's 14-diagonal storage.

    Returns (coef (14, N), b (N,), offsets).  coef[d, c] = A(c, c + offsets[d])
    after symmetric Dirichlet elimination (iterative_matrix.hpp:462-485).
    """
    node_id, n = numbering if numbering is not None else O.masked_numbering(prob)
    if n != node_id.size:
        raise ValueError("the 14-diagonal storage needs the full mesh (empty elements included)")
    offsets, _, _ = NS.band_offsets(prob)
    where = {int(o): d for d, o in enumerate(offsets)}
    ids, K, F, _, _ = O.element_terms(prob, T, thickness, node_id, n)
    coef = np.zeros((len(offsets), n))
    for (a, b), v in K.items():
        ra, rb = ids[a], ids[b]
        r = np.minimum(ra, rb)
        off = np.abs(ra - rb)
        d = where[int(off[0])] if off.size else 0
        coef[d, r] += v  # for one (a, b) pair every element hits a different entry
    Fv = np.zeros(n)
    for a in range(8):
        np.add.at(Fv, ids[a], F[a])
    is_d, vf, vl = O.dirichlet_values(prob, node_id, n)
    # b = F - A v_first on free rows, v_last on Dirichlet rows; zero Dirichlet rows/columns
    vD = np.where(is_d, vf, 0.0)
    y = coef[0] * vD
    for d in range(1, len(offsets)):
        o = int(offsets[d])
        y[:-o] += coef[d, :-o] * vD[o:]
        y[o:] += coef[d, :-o] * vD[:-o]
    b = Fv - y
    b[is_d] = vl[is_d]
    for d in range(1, len(offsets)):
        o = int(offsets[d])
        kill = is_d[:-o] | is_d[o:]
        coef[d, :-o][kill] = 0.0
    coef[0, is_d] = 1.0
    return coef, b, offsets


class IcCg:
    """IC(0)-PCG restatement with the reference's refactorisation cadence (every nfact solves)."""

    def __init__(self, maxit=1000, zeta=1e-6, nfact=10):
        self.lib = _iccg_lib()
        self.maxit, self.zeta, self.nfact = maxit, zeta, nfact
        self.ifact = 1
        self.u = None
        self.iters = 0
        self.err = 0.0
        self.status = 0

    def solve(self, coef, offsets, b, x0):
        nd, n = coef.shape
        self.ifact -= 1
        refactor = self.ifact == 0
        if self.ifact <= 0:
            self.ifact = self.nfact
        if self.u is None or self.u.size != coef.size:
            self.u = np.zeros(coef.size)
            refactor = True
        a = np.ascontiguousarray(coef.ravel())
        off = np.ascontiguousarray(offsets, np.int32)
        x = np.ascontiguousarray(x0, np.float64).copy()
        it, err = C.c_int(0), C.c_double(0.0)
        dp = C.POINTER(C.c_double)
        self.status = self.lib.oracle_iccg(n, nd, off.ctypes.data_as(C.POINTER(C.c_int)), a.ctypes.data_as(dp),
                                           self.u.ctypes.data_as(dp), 1 if refactor else 0,
                                           np.ascontiguousarray(b).ctypes.data_as(dp), x.ctypes.data_as(dp),
                                           self.maxit, self.zeta, C.byref(it), C.byref(err))
        self.iters, self.err = it.value, err.value
        return x


def sample(prob, cg_iterations=30, solver="port", zeta=1e-12):
    """Bounded sample of one outer loop of the reference's iterative Static3D.

    Times: the assembly (setMatrix + applyBC), one IC factorisation and
    ``cg_iterations`` preconditioned CG iterations.  Returns a dict of seconds.
    """
    numbering = O.masked_numbering(prob)
    th = O.element_thickness(prob)
    T = np.full(prob.shape, float(prob.inittemp))
    t0 = time.perf_counter()
    coef, b, offsets = assemble_diagonal(prob, T, th, numbering)
    t1 = time.perf_counter()
    x0 = O.from_full(numbering[0], numbering[1], T)
    if solver == "port":
        s = IcCg(maxit=0, zeta=zeta)
        s.solve(coef, offsets, b, x0)  # factorisation only
        t2 = time.perf_counter()
        s.ifact = 2  # reuse the factor
        s.maxit = cg_iterations
        s.solve(coef, offsets, b, x0)
        t3 = time.perf_counter()
        iters = s.iters
    else:
        raise ValueError(solver)
    return {"assembly_s": t1 - t0, "factor_s": t2 - t1, "cg_s": t3 - t2, "cg_iterations": iters,
            "per_iteration_s": (t3 - t2) / max(iters, 1), "nodes": int(b.size)}


def full_solve_iterative(prob, zeta=1e-12, maxit=5000, max_loops=30):
    """The whole outer k(T) loop of the reference's ``iterative`` algorithm with the IC(0)-PCG
    restatement on one core (therm3d.cpp:281-340 around iterative_matrix.hpp:141-339), timed.

    Returns wall seconds, outer loops, IC-CG iterations summed over the loops and the field."""
    numbering = O.masked_numbering(prob)
    th = O.element_thickness(prob)
    T = np.full(prob.shape, float(prob.inittemp))
    sv = IcCg(maxit=maxit, zeta=zeta)
    loops, iters = 0, 0
    t0 = time.perf_counter()
    while True:
        coef, b, offsets = assemble_diagonal(prob, T, th, numbering)
        x = sv.solve(coef, offsets, b, O.from_full(numbering[0], numbering[1], T))
        Tn = O.to_full(prob, numbering[0], x)
        err = float(np.max(np.abs(Tn - T)))
        T = Tn
        loops += 1
        iters += sv.iters
        if not ((sv.status != 0 or err > prob.maxerr) and loops < max_loops):
            break
    return {"wall_s": time.perf_counter() - t0, "loops": loops, "iterations": iters, "T": T}


def full_solve_cholesky(prob):
    """The whole outer loop of the reference's ``cholesky`` algorithm: the oracle's assembly and
    LAPACK dpbtrf/dpbtrs (cholesky_matrix.hpp:95,107) with the BLAS library's threads, timed."""
    t0 = time.perf_counter()
    T, toterr, rec = O.compute(prob)
    return {"wall_s": time.perf_counter() - t0, "loops": len(rec), "T": T}


def predict(sample_result, loops, iterations, nfact=10):
    """Seconds of a full iterative solve from a bounded sample: per loop an assembly, one IC
    factorisation per nfact solves (iterative_matrix.hpp:149-150), per iteration the sampled cost."""
    refactors = (loops + nfact - 1) // nfact
    return (loops * sample_result["assembly_s"] + refactors * sample_result["factor_s"]
            + iterations * sample_result["per_iteration_s"])
