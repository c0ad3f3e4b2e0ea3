"""Writes the golden fixture of the 128x128x200 layered case -- TEST INFRASTRUCTURE ONLY.

    python tests/golden/make_golden_c1.py           (about forty minutes on one core)
    python tests/golden/make_golden_c1.py 40,36,50  (a dry run on a smaller mesh, writes nothing)
    python tests/golden/make_golden_c1.py --refresh-inputs  (rewrite the stored input summary only)

The benchmark's case (``structures.layered_c1()``: seed 1000, 128 x 128 x 200 nodes,
anisotropic layers, convective top, Dirichlet bottom) solved by the reference's own
``iterative`` algorithm: NSPCG's IC-preconditioned CG compiled from the reference's
``extlib/nspcg`` into ``oracle/_ref`` (``make -C oracle ref``), driven to zeta = 1e-12 over
the full outer k(T) loop (therm3d.cpp:281-340), with the oracle's FP64 assembly into the
reference's 14-diagonal storage (iterative_matrix.hpp:373-393).

At this size the band Cholesky of the ``cholesky`` algorithm needs 433 GB and cannot run,
so the tight NSPCG solve is the reference answer.  The whole field (26 MB) is not stored:
the fixture keeps
  * a summary of the generated inputs (``input_summary``: axes, material table, a SHA-256 of
    the element materials, heat statistics, boundary conditions), so that a test regenerating
    the structure knows it has the problem the answers belong to;
  * the temperatures of 16384 seeded random nodes, of the whole plane through the hottest
    node and of the vertical line through it;
  * per outer loop: NSPCG iterations, err, max T, wall time and the FP64 relative residual
    ||b - A T|| / ||b|| of the linear system.
The per-loop record also goes to ``oracle/c1_iterations.json`` as ``nspcg:1e-12``.
"""
from __future__ import annotations

import hashlib
import json
import os
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import baseline as B  # noqa: E402
from oracle import characterize as CH  # noqa: E402
from oracle import fem3d as O  # noqa: E402
from oracle import nspcg as NS  # noqa: E402
from plask_gb300 import structures as S  # noqa: E402

OUT = HERE / "static3d_layered_c1_128x128x200_nspcg.npz"
N_RANDOM = 16384


def input_summary(s):
    """The solver inputs of a generated structure, in a form that survives the last-bit
    differences of libm between machines: the axes and the material table in full, a SHA-256
    of the (integer) element materials, the heat's nonzero count, sum and extremes, and the
    boundary conditions."""
    heat = np.asarray(s.heat, np.float64)
    return {"axes": [np.asarray(a, np.float64).tolist() for a in s.axes],
            "materials": {f: np.asarray(getattr(s, f), np.float64).tolist() for f in ("k300", "p", "kz_ratio", "hexp")},
            "empty": np.asarray(s.empty, bool).tolist(),
            "mat_sha256": hashlib.sha256(np.ascontiguousarray(s.mat, np.int32).tobytes()).hexdigest(),
            "heat": {"nonzero": int(np.count_nonzero(heat)), "sum": float(heat.sum()), "min": float(heat.min()),
                     "max": float(heat.max())},
            "bc": json.loads(json.dumps([s.temperature, s.heatflux, s.convection, s.radiation, s.maxerr,
                                         s.inittemp]))}


def inputs_match(s, summary, rtol=1e-12):
    """Whether a regenerated structure has the inputs a fixture's answers belong to."""
    now = input_summary(s)
    close = lambda a, b: np.allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=0)
    return (all(close(a, b) for a, b in zip(now["axes"], summary["axes"]))
            and all(close(now["materials"][f], summary["materials"][f]) for f in now["materials"])
            and now["empty"] == summary["empty"] and now["mat_sha256"] == summary["mat_sha256"]
            and now["heat"]["nonzero"] == summary["heat"]["nonzero"]
            and all(close(now["heat"][f], summary["heat"][f]) for f in ("sum", "min", "max"))
            and now["bc"] == summary["bc"])


def sample_nodes(shape, rng):
    """Canonical node indices (k, j, i flattened) of the stored random subset."""
    n = int(np.prod(shape))
    return np.sort(rng.choice(n, size=min(N_RANDOM, n), replace=False))


def main(size=None):
    """size: a smaller (n0, n1, n2) for a dry run that writes nothing."""
    if not NS.available():
        raise SystemExit("oracle/_ref/libnspcg_ref.so is not built: make -C oracle ref (needs the reference tree)")
    s = S.layered_c1() if size is None else S.layered_c1(n=size)
    summary = input_summary(s)
    prob = O.from_structure(s, empty_elements="include")
    numbering = O.masked_numbering(prob)
    node_id, n_active = numbering
    th = O.element_thickness(prob)
    T = np.full(prob.shape, float(prob.inittemp))
    sv = NS.NspcgSolver(prob, maxit=5000, zeta=1e-12)
    loops, toterr = [], 0.0
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        coef, b, off = B.assemble_diagonal(prob, T, th, numbering)
        A = CH.build_matrix(coef, off)
        t1 = time.perf_counter()
        x = sv.solve(A, b, O.from_full(node_id, n_active, T))
        t2 = time.perf_counter()
        relres = float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
        Tn = O.to_full(prob, node_id, x)
        err = float(np.max(np.abs(Tn - T)))
        toterr = max(toterr, err)
        T = Tn
        loops.append({"iterations": sv.iters, "converged": sv.ier != 1, "err": err, "maxT": float(T.max()),
                      "assembly_s": t1 - t0, "solve_s": t2 - t1, "rel_residual": relres})
        print(loops[-1], flush=True)
        if not ((sv.ier == 1 or err > prob.maxerr) and len(loops) < 30):
            break
    wall = time.perf_counter() - t_start
    rng = np.random.default_rng(20261204)
    idx = sample_nodes(prob.shape, rng)
    Tf = T.ravel()
    k_hot, j_hot, i_hot = np.unravel_index(int(np.argmax(Tf)), prob.shape)
    plane = np.ascontiguousarray(T[k_hot])
    line = np.ascontiguousarray(T[:, j_hot, i_hot])
    meta = {"generator": "structures.layered_c1(seed=1000, n=(128, 128, 200))", "inputs": summary,
            "solver": "NSPCG ic + cg from extlib/nspcg, zeta 1e-12, maxit 5000, nfact 10", "order": prob.order,
            "loops": loops, "toterr": toterr, "rel_residual": loops[-1]["rel_residual"],
            "max_t": float(Tf.max()), "hot_node": [int(k_hot), int(j_hot), int(i_hot)], "wall_s": wall,
            "cores": 1, "cpu_count": os.cpu_count()}
    if size is not None:
        print("dry run:", {k: meta[k] for k in ("toterr", "rel_residual", "max_t", "hot_node", "wall_s")})
        return
    np.savez_compressed(OUT, meta=np.array(json.dumps(meta)), idx=idx, T_idx=Tf[idx], plane=plane, line=line)
    print("wrote", OUT, "wall", wall)
    res = json.loads(CH.OUT.read_text()) if CH.OUT.exists() else {}
    res["nspcg:1e-12"] = {"solver": "nspcg", "zeta": 1e-12, "maxit": 5000, "loops": loops, "wall_s": wall}
    CH.OUT.write_text(json.dumps(res, indent=1))


def refresh_inputs():
    """Rewrite the input summary of the existing fixture (the answers are kept)."""
    d = dict(np.load(OUT))
    meta = json.loads(str(d["meta"]))
    meta.pop("input_sha256", None)
    meta["inputs"] = input_summary(S.layered_c1())
    d["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **d)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--refresh-inputs":
        refresh_inputs()
    else:
        main(tuple(int(v) for v in sys.argv[1].split(",")) if len(sys.argv) > 1 else None)
