#!/usr/bin/env python
"""Static3D time-to-solution benchmark on the 128x128x200 layered structure.

One step = one full ``Static3D.compute()`` of the scaled layered case
(128x128x200 nodes = 3.28 M unknowns, 12 layers with anisotropic k(T) on a
150 um substrate, 4 um disc source at 1e16 W/m^3, bottom at 300 K, convective
top h = 10 W/m^2K): the outer k(T) loop from 300 K to maxerr = 0.05 K with
every linear solve taken to an FP64 relative residual of 1e-14 (max |dT| <=
1e-6 K against the FP64 oracle, checked by the parity tests).

value    solves/s over K timed steps, device time (CUDA events on the solver's
         stream), inputs resident in HBM, L2 flushed before every step;
e2e      the same through the C ABI with pinned host buffers: upload of the
         element materials, heat and boundary nodes, compute, download of T;
plain    the plain FP64 Jacobi-PCG solver on the same case, for comparison;
roofline the operator kernel (matrix-free stiffness apply, FP32) timed with
         CUDA events over 20 launches with L2 flushed before each launch;
parity   max |dT| of the final field against the reference's own NSPCG solution
         (zeta 1e-12, tests/golden/static3d_layered_c1_128x128x200_nspcg.npz) at
         16384 seeded nodes, the plane and the vertical line through the hottest
         node, and the FP64 relative residuals of both;
learned  the learned preconditioner on a structure of its own configuration
         (structures.learned_c2, seed 2001, 124x108x128): learned flexible CG + mixed
         precision, Jacobi-PCG mixed precision and plain FP64, with iterations, the
         network's device time and max |dT| between them;
coupled  the thermo-electric loop at 200x200x120 (structures.shockley_c4), per round;
sweep    64 structures of the uneven-size sweep, batched and one at a time;
cpu_baseline  the reference's default iterative algorithm (IC + CG) restated
         on the host (oracle), timed on a bounded sample of the 128x128x200 case
         and extrapolated with the reference NSPCG's own iteration counts; beside
         it the 40x40x60 configuration solved in full on the host, with the band
         Cholesky (all cores) and with IC-CG (one core), and the extrapolation
         model's prediction for that solve.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload sweep [--sweep-count 256]   # batched sweep line (not the default)

The sweep line solves the uneven-size sweep (layered generator, 32..96 nodes per
axis, source power 1e15..1e16 W/m^3): every structure one at a time, then all of
them batched (concurrent solves on separate streams) with the thread count and
stencil grid policy the autotuner picks on a sample of 32 structures.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Static3D time-to-solution & solves/s at |dT|<=1e-6 K (layered 128x128x200, mixed FP32/FP64 vs plain FP64 GPU)"
UNIT = "solves/s"
WORKLOAD = "layered-aniso-128x128x200 (3.28M nodes, convective top), full outer k(T) loop to maxerr 0.05 K, rtol 1e-14"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--algorithm", default="gpu-mixed")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--cpu-iterations", type=int, default=10, help="CG iterations in the CPU baseline sample")
    ap.add_argument("--size", default="128,128,200")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-coupled", action="store_true", help="skip the coupled thermo-electric record")
    ap.add_argument("--no-sweep", action="store_true", help="skip the batched-sweep record")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner record")
    ap.add_argument("--learned-weights", default=None, help="weights file of the learned record (default: shipped)")
    ap.add_argument("--learned-seed", type=int, default=2001)
    ap.add_argument("--sweep-record-count", type=int, default=64)
    ap.add_argument("--sweep-record-sequential", type=int, default=8)
    ap.add_argument("--workload", default="layered", choices=["layered", "sweep"])
    ap.add_argument("--sweep-count", type=int, default=256)
    ap.add_argument("--sweep-loops", type=int, default=30, help="outer-loop cap of every sweep solve")
    ap.add_argument("--clocks-dir", default=None, help="directory that keeps the raw nvidia-smi clock samples")
    ap.add_argument("--operator-only", action="store_true",
                    help="only set up the case and time the operator kernel (for kernel profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-reduction across ranks (gloo on the host; the path itself has no collective)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, directory=None):
        self.gpu = gpu_index
        self.proc = None
        # the raw samples go to `directory` when given (kept), else to a temporary file
        if directory:
            self.path = pathlib.Path(directory) / f"clocks_rank{gpu_index}.csv"
        else:
            import tempfile

            self.path = pathlib.Path(tempfile.mkdtemp(prefix="plgpu_clocks_")) / f"clocks_rank{gpu_index}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the operator kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "operator_traffic.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return d
        except Exception:
            return None
    return None


# ------------------------------------------------------------------------------------------
# CPU baseline (the reference's default iterative path restated on the host)


def baseline_problem(size):
    """The bench case as the oracle's problem (the reference's iterative algorithm includes
    empty elements, fem_solver.hpp:182-189)."""
    from oracle import fem3d as O
    from plask_gb300 import structures as S

    return O.from_structure(S.layered_c1(n=size), empty_elements="include")


def c1_iteration_record(size):
    """(outer loops, IC-CG iterations, note) of the reference's iterative solve at zeta 1e-12."""
    char_path = ROOT / "oracle" / "c1_iterations.json"
    if char_path.exists() and tuple(size) == (128, 128, 200):
        ch = json.loads(char_path.read_text())
        # the reference's own NSPCG first (5641 iterations); the IC(0) port converges in fewer
        key = next((k for k in ("nspcg:1e-12", "port:1e-12") if k in ch), None)
        if key:
            lp = ch[key]["loops"]
            iters = sum(x["iterations"] for x in lp)
            return len(lp), iters, (f"{len(lp)} outer loops and {iters} IC-CG iterations in total at zeta 1e-12 "
                                    f"({key}, oracle/c1_iterations.json)")
    return 5, 5 * 1000, "assumed 5 outer loops of 1000 iterations (reference maxit)"


def cpu_baseline(size, cg_iterations, prob=None):
    from oracle import baseline as B

    if prob is None:
        prob = baseline_problem(size)
    r = B.sample(prob, cg_iterations=cg_iterations)
    loops, iters, note = c1_iteration_record(size)
    est = B.predict(r, loops, iters)
    return {
        "value": 1.0 / est,
        "unit": UNIT,
        "cores": 1,
        "kind": "port",
        "sample": (f"one outer loop of the 128x128x200 case on 1 host core: numpy assembly into the reference's "
                   f"14-diagonal storage {r['assembly_s']:.2f} s, IC(0) factorisation {r['factor_s']:.2f} s, "
                   f"{r['cg_iterations']} CG iterations at {r['per_iteration_s']:.3f} s; extrapolated with {note} "
                   f"to {est:.0f} s per solve (NSPCG is single-threaded in the reference)"),
        "seconds_per_solve": est,
    }


def cpu_c0_measured():
    """The 40x40x60 configuration (layered_c0, seed 1) solved in full on the host, both reference
    algorithms, with the extrapolation model's prediction of the iterative solve beside it."""
    import numpy as np

    from oracle import baseline as B
    from oracle import fem3d as O
    from plask_gb300 import structures as S

    s = S.layered_c0(seed=1)
    p_it = O.from_structure(s, empty_elements="include")
    it = B.full_solve_iterative(p_it)
    sm = B.sample(p_it, cg_iterations=50)
    pred = B.predict(sm, it["loops"], it["iterations"])
    ch = B.full_solve_cholesky(O.from_structure(s))
    return {
        "workload": "layered-40x40x60 (seed 1), full outer loop to maxerr 0.05 K",
        "cpu": _cpu_model(), "nproc": os.cpu_count(),
        "measured_c0_s": {"cholesky": ch["wall_s"], "iterative": it["wall_s"]},
        "cores": {"cholesky": os.cpu_count(), "iterative": 1},
        "iterative_loops": it["loops"], "iterative_iterations": it["iterations"],
        "cholesky_loops": ch["loops"],
        "predicted_c0_s": pred,
        "prediction_over_measured": pred / it["wall_s"],
        "max_dT_iterative_vs_cholesky_K": float(np.max(np.abs(it["T"] - ch["T"]))),
    }


def _cpu_model():
    try:
        for line in pathlib.Path("/proc/cpuinfo").read_text().splitlines():
            low = line.lower()
            if low.startswith("model name") or low.startswith("cpu part"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def reference_parity(T, rel_residual):
    """max |dT| of a canonical (n2, n1, n0) field against the reference NSPCG golden field."""
    import numpy as np

    path = ROOT / "tests" / "golden" / "static3d_layered_c1_128x128x200_nspcg.npz"
    if not path.exists() or T.shape != (200, 128, 128):
        return None
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    k, j, i = meta["hot_node"]
    dT = max(float(np.max(np.abs(T.ravel()[d["idx"]] - d["T_idx"]))), float(np.max(np.abs(T[k] - d["plane"]))),
             float(np.max(np.abs(T[:, j, i] - d["line"]))))
    return {"reference": "NSPCG (ic + cg from the reference's extlib/nspcg) at zeta 1e-12, 5 outer loops",
            "fixture": "tests/golden/static3d_layered_c1_128x128x200_nspcg.npz",
            "compared_nodes": int(d["idx"].size + d["plane"].size + d["line"].size),
            "max_dT_vs_reference_K": dT, "rel_residual_fp64": rel_residual,
            "reference_rel_residual_fp64": meta["rel_residual"], "reference_max_t_K": meta["max_t"]}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    size = tuple(int(v) for v in args.size.split(","))
    prob = baseline_problem(size)
    for _ in range(args.warmup):  # untimed samples of the same work
        cpu_baseline(size, args.cpu_iterations, prob)
    vals, times = [], []
    last = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        last = cpu_baseline(size, args.cpu_iterations, prob)
        times.append(time.perf_counter() - t0)
        vals.append(last["value"])
    v = statistics.median(vals)
    c0 = None
    if not args.no_cpu:
        try:
            c0 = cpu_c0_measured()
        except Exception as e:  # reported, not required
            c0 = {"failed": str(e)}
    out = {
        "metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded layered generator)",
        "config": {"workload": WORKLOAD, "nodes": int(size[0] * size[1] * size[2]), "l2": "host run, n/a"},
        "cpu_baseline": dict({k: last[k] for k in ("value", "unit", "cores", "kind", "sample")}, c0_measured=c0),
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


# ------------------------------------------------------------------------------------------
# GPU arm


def coupled_record():
    """The coupled thermo-electric loop (thermoelectric.py:181-219) at 200x200x120
    (structures.shockley_c4(seed=4000)): electrical compute(tfreq), its Joule heat to the
    thermal solver on the device, thermal compute(1), until both errors are within maxerr;
    each call timed (host clock around synchronised calls)."""
    import numpy as np
    import torch

    from plask_gb300 import electrical as EL
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    s = S.shockley_c4(seed=4000)
    te = EL.ThermoElectric3D()
    te.thermal = TH.solver_for_structure(s.thermal, ordering="best", algorithm="gpu-mixed")
    te.electrical = EL.solver_for_structure(s, ordering="best", algorithm="gpu-mixed")
    te.reconnect()
    te.invalidate()
    te.initialize()
    torch.cuda.synchronize()
    rounds = []
    verr, terr = 2.0 * te.electrical.maxerr, 2.0 * te.thermal.maxerr
    t_start = time.perf_counter()
    while terr > te.thermal.maxerr or verr > te.electrical.maxerr:
        t0 = time.perf_counter()
        verr = te.electrical.compute(te.tfreq)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        te._move_heat()
        terr = te.thermal.compute(1)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        es, ts = te.electrical.stats, te.thermal.stats
        rounds.append({"electrical_s": t1 - t0, "electrical_loops": es.get("loops"),
                       "electrical_cg_iterations": es.get("inner_iterations"), "verr_pct": verr,
                       "thermal_s": t2 - t1, "thermal_cg_iterations": ts.get("inner_iterations"), "terr_K": terr})
        if len(rounds) >= 30:
            break
    wall = time.perf_counter() - t_start
    n = [len(a) for a in s.axes]
    return {"workload": f"coupled thermo-electric loop, shockley_c4 seed 4000, {n[0]}x{n[1]}x{n[2]} nodes, "
                        f"{max(v for _, v in s.voltage):.3f} V on a 6 um top contact, maxerr 0.05 K / 0.1 %",
            "seconds": wall, "rounds": len(rounds), "per_round": rounds,
            "electrical_s": sum(r["electrical_s"] for r in rounds), "thermal_s": sum(r["thermal_s"] for r in rounds),
            "total_current_mA": float(te.get_total_current()), "max_t_K": float(te.thermal.stats.get("max_t", np.nan)),
            "electrical_operator": "k_apply_tma" if n[0] % 4 == 0 and n[0] <= 256 else "k_apply_shared"}


def sweep_record(count, sequential, algorithm="gpu-mixed", loops=30):
    """A subset of the batched sweep (uneven layered structures, 32..96 nodes per axis): the
    autotuner on the first 16, all ``count`` solved batched, the first ``sequential`` one at a
    time (the reference's way), and their agreement."""
    import numpy as np
    import torch

    from plask_gb300 import _native
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    structs = S.sweep_c3(count=count)
    svs = []
    for st in structs:
        sv = TH.solver_for_structure(st, ordering="best", algorithm=algorithm)
        sv.initialize()
        svs.append(sv)
    fems = [sv._fem for sv in svs]
    nodes = int(sum(np.prod(st.shape) for st in structs))
    seq = fems[:sequential]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for f in seq:
        f.compute(loops)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    T_seq = [f.temperature() for f in seq]
    threads, share, trials = _native.batch_tune(fems[: min(16, len(fems))], loops=loops, max_threads=32)
    for f in fems:
        f.set_grid_share(share)
        f.invalidate()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, bstats, _ = _native.batch_compute(fems, loops=loops, threads=threads)
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    node_iters = float(sum(int(np.prod(st.shape)) * b["inner_iterations"] for st, b in zip(structs, bstats)))
    dT = max(float(np.max(np.abs(fems[k].temperature() - T_seq[k]))) for k in range(len(seq)))
    return {"workload": f"{count} structures of the uneven-size sweep (seed 3000: 32..96 nodes per axis, "
                        f"{nodes} nodes in total, 1e15..1e16 W/m^3, at most {loops} outer loops)",
            "batched_solves_per_s": count / t_bat, "batched_seconds": t_bat, "threads": threads, "grid_share": share,
            "one_at_a_time_solves_per_s": sequential / t_seq, "one_at_a_time_sample": sequential,
            "speedup": (count / t_bat) / (sequential / t_seq),
            "cg_iterations": int(sum(b["inner_iterations"] for b in bstats)),
            "batched_node_iterations_per_us": node_iters / (t_bat * 1e6),
            "max_dT_batched_vs_one_at_a_time_K": dT}


def learned_record(weights=None, seed=2001):
    """The learned preconditioner on a structure of its own family (structures.learned_c2,
    not one of the training seeds): the learned flexible CG inside the mixed-precision
    refinement (gpu-learned), the Jacobi-PCG mixed solve (gpu-mixed) and plain FP64
    Jacobi-PCG (gpu-pcg), each a full compute() from 300 K (device time of the second of
    two runs), with CG iterations (those of the learned flexible CG and those of the
    Jacobi-PCG that finishes a correction after a fallback), the device time of one network
    forward pass and of one preconditioner application, and max |dT| against the plain
    FP64 answer."""
    import numpy as np

    from plask_gb300 import learned as LN
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    path = pathlib.Path(weights) if weights else LN.WEIGHTS_C2
    net = LN.load_c2(path)
    s = S.learned_c2(seed=seed)

    def run(algo, reps):
        for _ in range(reps):
            sv = TH.solver_for_structure(s, algorithm=algo)
            if algo == "gpu-learned":
                sv.preconditioner = net
            sv.compute()
        st = sv.stats
        rec = {"s_per_solve": st["total_ms"] / 1e3, "solves_per_s": 1e3 / st["total_ms"], "outer_loops": st["loops"],
               "cg_iterations": st["inner_iterations"], "us_per_iteration": 1e3 * st["total_ms"] / st["inner_iterations"]}
        if algo == "gpu-learned":
            rec["fallbacks"] = st.get("fallbacks")
            rec["learned_fcg_iterations"] = st.get("learned_iterations")
            rec["jacobi_fallback_iterations"] = st["inner_iterations"] - st.get("learned_iterations", 0)
            fwd, app = net.time_apply(sv._fem, reps=20)
            rec["network_forward_us"] = 1e3 * fwd
            rec["preconditioner_apply_us"] = 1e3 * app
        return rec, sv._full_temperature()

    plain, T_plain = run("gpu-pcg", 1)
    mixed, T_mixed = run("gpu-mixed", 2)
    learned, T_learned = run("gpu-learned", 2)
    mixed["max_dT_vs_plain_fp64_K"] = float(np.nanmax(np.abs(T_mixed - T_plain)))
    learned["max_dT_vs_plain_fp64_K"] = float(np.nanmax(np.abs(T_learned - T_plain)))
    learned["max_dT_vs_jacobi_mixed_K"] = float(np.nanmax(np.abs(T_learned - T_mixed)))
    n = [len(a) for a in s.axes]
    return {"workload": f"learned_c2 seed {seed}: {n[0]}x{n[1]}x{n[2]} nodes, {len(s.k300)} materials, etched mesa, "
                        f"oxide aperture at 1e-2, Gaussian heat blobs; bottom 300 K, maxerr {s.maxerr} K",
            "weights": f"{path.name}: 4-level U-Net trained on {len(LN.TRAIN_SEEDS) * LN.STEPS_PER_STRUCTURE} "
                       f"residual->error pairs from {len(LN.TRAIN_SEEDS)} learned_c2 structures",
            "learned": learned, "jacobi_mixed": mixed, "plain_fp64": plain,
            "learned_speedup_vs_plain_fp64": plain["s_per_solve"] / learned["s_per_solve"],
            "jacobi_mixed_speedup_vs_plain_fp64": plain["s_per_solve"] / mixed["s_per_solve"],
            "learned_speedup_vs_jacobi_mixed": mixed["s_per_solve"] / learned["s_per_solve"]}


def run_sweep(args):
    """Batched sweep: one-at-a-time vs concurrent solves of the uneven-size sweep."""
    # more hardware work queues than the default 8, so that up to 32 solver streams
    # do not alias onto shared queues (read when the CUDA context is created)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import numpy as np
    import torch

    from plask_gb300 import _native
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH

    torch.cuda.set_device(0)
    structs = S.sweep_c3(count=args.sweep_count)
    svs = []
    for s in structs:
        sv = TH.solver_for_structure(s, ordering="best", algorithm=args.algorithm)
        sv.initialize()
        svs.append(sv)
    fems = [sv._fem for sv in svs]
    nodes = int(sum(np.prod(s.shape) for s in structs))
    # one at a time (the reference's way: one solver object after another)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    iters = 0
    unconverged, failed = [], []
    for k, f in enumerate(fems):
        try:
            _, st = f.compute(args.sweep_loops)
        except _native.ComputationError:  # a runaway structure whose solve breaks down
            failed.append(k)
            unconverged.append(k)
            continue
        iters += st["inner_iterations"]
        if st["err"] > 0.05 or not st["converged"]:
            unconverged.append(k)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    T_seq = [f.temperature() for f in fems]
    # autotune on a sample, then the whole sweep batched
    sample = [f for k, f in enumerate(fems) if k not in failed][: min(32, len(fems))]
    threads, share, trials = _native.batch_tune(sample, loops=args.sweep_loops, max_threads=32)
    for f in fems:
        f.set_grid_share(share)
        f.invalidate()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    try:
        _native.batch_compute(fems, loops=args.sweep_loops, threads=threads)
    except _native.ComputationError:  # every solve has run; the runaway ones are counted above
        pass
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    # solves that did not settle within the loop cap (thermal runaway) follow different
    # trajectories under different grids; compare the settled ones
    dT = max(float(np.max(np.abs(fems[k].temperature() - T_seq[k])))
             for k in range(len(fems)) if k not in unconverged)
    out = {
        "metric": "batched sweep solves/s (uneven layered structures, 32..96 nodes per axis)",
        "value": len(fems) / t_bat, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
        "dtype": "f32 inner CG, f64 refinement", "data": "synthetic (seeded sweep generator, seed 3000)",
        "config": {"workload": f"sweep of {len(fems)} layered structures, {nodes} nodes in total, "
                               f"source power 1e15..1e16 W/m^3, at most {args.sweep_loops} outer loops per solve",
                   "algorithm": args.algorithm},
        "one_at_a_time": {"solves_per_s": len(fems) / t_seq, "seconds": t_seq, "cg_iterations": iters,
                          "solves_not_within_maxerr": len(unconverged),
                          "solves_broken_down": len(failed)},
        "batched": {"seconds": t_bat, "threads": threads, "grid_share": share,
                    "speedup_vs_one_at_a_time": t_seq / t_bat},
        "tuner_trials_solves_per_s": [float(v) for v in trials],
        "max_dT_batched_vs_one_at_a_time_K": dT,
        "max_dT_note": "over the solves that settled within the loop cap",
    }
    print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    # more hardware work queues than the default 8 for the batched sweep's solver streams
    # (read when the CUDA context is created)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if args.workload == "sweep":
        return run_sweep(args)
    dist = Dist()
    import numpy as np
    import torch

    torch.cuda.set_device(dist.local)
    from plask_gb300 import _native
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH
    from plask_gb300.mesh import to_mesh_order

    size = tuple(int(v) for v in args.size.split(","))
    s = S.layered_c1(n=size)
    sv = TH.solver_for_structure(s, ordering="best", algorithm=args.algorithm)
    sv.initialize()
    fem = sv._fem
    stream = torch.cuda.ExternalStream(fem.stream())
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    if args.operator_only:
        ms, by = fem.time_operator(32, reps=3, flush_l2=True)
        ms64, by64 = fem.time_operator(64, reps=2, flush_l2=True)
        print(json.dumps({"operator_fp32_ms": ms, "bytes": by, "gbs": by / ms / 1e6,
                          "operator_fp64_ms": ms64, "bytes64": by64, "nodes": int(np.prod(size))}))
        return 0

    def step():
        fem.invalidate()
        fem.set_solver(args.algorithm, sv.rtol, 0, "warning", "default", True)
        _, st = fem.compute(0)
        return st

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(dist.local, args.clocks_dir)
    sampler.start()
    dist.barrier()
    torch.cuda.synchronize()
    times, stats = [], []
    for _ in range(args.steps):
        flush.fill_(1)  # evict the previous step's working set from L2
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        stats.append(st)
    torch.cuda.synchronize()
    dist.barrier()
    clocks = sampler.stop()
    t_total = dist.max(sum(times))
    solves = dist.sum(len(times))
    value = solves / t_total
    T_mixed = fem.temperature()
    parity = reference_parity(sv._full_temperature(), stats[-1]["last_rel_residual"])

    # end to end through the C ABI: pinned host inputs, results read back every step
    mat_h = torch.from_numpy(to_mesh_order(s.mat, sv.mesh.ordering).astype(np.int32)).pin_memory()
    heat_h = torch.from_numpy(to_mesh_order(s.heat, sv.mesh.ordering).astype(np.float64)).pin_memory()
    bc_nodes = [(_native.BC_TEMPERATURE, TH.RectangularMesh3D.Bottom().nodes(sv.mesh), 300.0, 0.0),
                (_native.BC_CONVECTION, TH.RectangularMesh3D.Top().nodes(sv.mesh), 10.0, 300.0)]
    bc_h = [(k, torch.from_numpy(n.astype(np.int64)).pin_memory(), a, b) for k, n, a, b in bc_nodes]
    nn, ne = fem.sizes()
    T_h = torch.empty(nn, dtype=torch.float64).pin_memory()
    h2d = mat_h.numel() * 4 + heat_h.numel() * 8 + sum(x[1].numel() * 8 for x in bc_h)
    d2h = T_h.numel() * 8
    e2e_times = []
    dist.barrier()
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fem.set_elements(mat_h.numpy(), heat_h.numpy())
        for kind in range(4):
            fem.clear_bc(kind)
        for k, nodes, a, b in bc_h:
            fem.add_bc(k, nodes.numpy(), a, b)
        fem.set_solver(args.algorithm, sv.rtol, 0, "warning", "default", True)
        fem.compute(0)
        fem.temperature(out=T_h.numpy())
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = solves / dist.max(sum(e2e_times))

    # plain FP64 Jacobi-PCG on the same case
    plain = None
    if args.plain_steps > 0:
        pt, pit = [], []
        for _ in range(args.plain_steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            fem.invalidate()
            fem.set_solver("gpu-pcg", sv.rtol, 0, "warning", "default", True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, st = fem.compute(0)
            e1.record(stream)
            e1.synchronize()
            pt.append(e0.elapsed_time(e1) / 1e3)
            pit.append(st["inner_iterations"])
        T_plain = fem.temperature()
        plain = {"solves_per_s": len(pt) / sum(pt), "s_per_solve": statistics.mean(pt), "cg_iterations": pit[-1],
                 "max_dT_vs_mixed_K": float(np.max(np.abs(T_plain - T_mixed))),
                 "speedup_of_value": (len(pt) / sum(pt)) and value / (len(pt) / sum(pt))}

    # operator roofline (FP32 stiffness apply, L2 flushed before each launch)
    ms, by = fem.time_operator(32, reps=20, flush_l2=True)
    ms_l2, _ = fem.time_operator(32, reps=20, flush_l2=False)
    ms64, by64 = fem.time_operator(64, reps=5, flush_l2=True)
    peak, peak_kind = measured_peaks()
    achieved = by / (ms * 1e-3) / 1e9
    tr = profiled_traffic()
    roofline = {"kernel": "k_apply_tma (FP32 matrix-free stiffness apply of the inner CG: TMA-staged planes, "
                          "packed f32x2 arithmetic)", "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} hbm_gbs", "bytes_per_launch": by, "ms_per_launch": ms,
                "traffic": (tr or {}).get("bytes_per_launch"),
                "l2_resident_ms_per_launch": ms_l2,
                "fp64_ms_per_launch": ms64, "fp64_achieved_gbs": by64 / (ms64 * 1e-3) / 1e9}

    coupled = sweep = learned = None
    if dist.rank == 0 and not args.no_learned:
        try:
            learned = learned_record(args.learned_weights, args.learned_seed)
        except Exception as e:  # reported, not required
            learned = {"failed": str(e)}
    if dist.rank == 0 and not args.no_coupled:
        try:
            coupled = coupled_record()
        except Exception as e:  # reported, not required
            coupled = {"failed": str(e)}
    if dist.rank == 0 and not args.no_sweep:
        try:
            sweep = sweep_record(args.sweep_record_count, args.sweep_record_sequential, args.algorithm)
        except Exception as e:
            sweep = {"failed": str(e)}

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(size, args.cpu_iterations)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}
        try:
            cpu["c0_measured"] = cpu_c0_measured()
        except Exception as e:
            cpu["c0_measured"] = {"failed": str(e)}

    last = stats[-1]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner CG, f64 refinement",
        "data": "synthetic (seeded layered generator, seed 1000)",
        "config": {"workload": WORKLOAD, "algorithm": args.algorithm, "nodes": int(np.prod(size)),
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": f"replicas x{dist.world}"},
        "solve": {"outer_loops": last["loops"], "cg_iterations": last["inner_iterations"],
                  "refinements": last["refinements"], "rel_residual": last["last_rel_residual"],
                  "max_t_K": last["max_t"], "toterr_K": last["toterr"]},
        "plain_fp64": plain,
        "parity": parity,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": 1e3 * statistics.mean(e2e_times)},
        "gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
        "roofline": roofline,
        "learned": learned,
        "coupled": coupled,
        "sweep": sweep,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if dist.rank == 0:
        print(json.dumps(out))
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
