"""Iteration counts of the reference's iterative Static3D on the scaled layered case -- TEST INFRASTRUCTURE.

Runs the full outer k(T) loop of the reference's default algorithm (IC + CG,
refactorisation every 10 solves) on the 128x128x200 layered case with the
oracle's assembly and either NSPCG built from the reference tree ("nspcg") or
the oracle's IC(0)-PCG restatement ("port"), at the reference's default
stopping value zeta = 1e-6 and at zeta = 1e-12.  The per-loop iteration counts
are written to oracle/c1_iterations.json; the CPU baseline of the benchmark
extrapolates its bounded sample with them.

    python -m oracle.characterize [nspcg|port] [zeta ...]
"""
import json
import pathlib
import sys
import time

import numpy as np

from . import baseline as B
from . import fem3d as O
from . import nspcg as NS

OUT = pathlib.Path(__file__).resolve().parent / "c1_iterations.json"


def run(solver, zeta, maxit=1000, max_loops=12):
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parents[1]))
    from plask_gb300 import structures as S

    s = S.layered_c1()
    prob = O.from_structure(s, empty_elements="include")
    numbering = O.masked_numbering(prob)
    th = O.element_thickness(prob)
    T = np.full(prob.shape, 300.0)
    sv = B.IcCg(maxit=maxit, zeta=zeta) if solver == "port" else NS.NspcgSolver(prob, maxit=maxit, zeta=zeta)
    loops = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        coef, b, off = B.assemble_diagonal(prob, T, th, numbering)
        t1 = time.perf_counter()
        x0 = O.from_full(numbering[0], numbering[1], T)
        if solver == "port":
            x = sv.solve(coef, off, b, x0)
            its, conv = sv.iters, sv.status == 0
        else:
            # NSPCG takes the eliminated matrix; rebuild it from the diagonal storage
            x = _nspcg_solve(sv, coef, off, b, x0)
            its, conv = sv.iters, sv.ier != 1
        t2 = time.perf_counter()
        Tn = O.to_full(prob, numbering[0], x)
        err = float(np.max(np.abs(Tn - T)))
        T = Tn
        loops.append({"iterations": its, "converged": bool(conv), "err": err, "maxT": float(T.max()),
                      "assembly_s": t1 - t0, "solve_s": t2 - t1})
        print(solver, zeta, loops[-1], flush=True)
        if not ((not conv or err > prob.maxerr) and len(loops) < max_loops):
            break
    return {"solver": solver, "zeta": zeta, "maxit": maxit, "loops": loops, "wall_s": time.perf_counter() - t_start}


def build_matrix(coef, off):
    """The symmetric CSR matrix of the reference's 14-diagonal storage coef[d, c] = A(c, c + off[d])."""
    import scipy.sparse as sp

    nd, n = coef.shape
    diags = [coef[0]]
    offs = [0]
    for d in range(1, nd):
        o = int(off[d])
        diags += [coef[d, :-o], coef[d, :-o]]
        offs += [o, -o]
    return sp.diags(diags, offs, shape=(n, n), format="csr")


def _nspcg_solve(sv, coef, off, b, x0):
    # NSPCG takes the eliminated matrix; rebuild it from the diagonal storage
    return sv.solve(build_matrix(coef, off), b, x0)


if __name__ == "__main__":
    solver = sys.argv[1] if len(sys.argv) > 1 else "port"
    zetas = [float(z) for z in sys.argv[2:]] or [1e-6, 1e-12]
    res = json.loads(OUT.read_text()) if OUT.exists() else {}
    for z in zetas:
        r = run(solver, z)
        res[f"{solver}:{z:g}"] = r
        OUT.write_text(json.dumps(res, indent=1))
