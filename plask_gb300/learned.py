"""Training recipe and trained weights of the learned preconditioner.

The network (:class:`plask_gb300._native.UNet`, include/plgpu_unet.h) is trained on
the GPU by its own forward and backward kernels on residual -> error pairs that the
FEM of a training structure generates (a random smooth error e, r = A e).  The recipe
here trains it for the learned-preconditioner family of structures
(:func:`plask_gb300.structures.learned_c2`: 8-40 random layers, an etched cylindrical
mesa, an annular oxide aperture at 1e-2 of its host layer's conductivity, 96..160
nodes per axis, 1-3 Gaussian heat blobs): ten training structures (seeds 2100..2109,
disjoint from the evaluation seeds 2000..2099), 2000 pairs on each, 20 000 pairs.

The weights it produced are shipped as ``data/unet_c2.bin`` (the weights file
format of ``plgpu_unet_save``: header, FP32 weights, checksum).

    python -m plask_gb300.learned [--out PATH] [--steps 2000] [--pairs jacobi]
    python -m plask_gb300.learned --time SEED   # device time of the shipped network on learned_c2(SEED)
"""
from __future__ import annotations

import argparse
import pathlib
import time

WEIGHTS_C2 = pathlib.Path(__file__).resolve().parent / "data" / "unet_c2.bin"
TRAIN_SEEDS = tuple(range(2100, 2110))
STEPS_PER_STRUCTURE = 2000


def train_c2(net=None, seeds=TRAIN_SEEDS, steps=STEPS_PER_STRUCTURE, lr=1e-3, smooth=(5, 60), pairs="jacobi",
             net_seed=11, log=print):
    """Train ``net`` (a new UNet(net_seed) when None) on ``steps`` pairs of each structure
    learned_c2(seed) for seed in ``seeds``; returns (net, [(seed, first-50 mean loss,
    last-200 mean loss)])."""
    import numpy as np

    from . import _native
    from . import structures as S
    from . import thermal as TH

    if net is None:
        net = _native.UNet(seed=net_seed)
    summary = []
    for j, seed in enumerate(seeds):
        s = S.learned_c2(seed=seed)
        sv = TH.solver_for_structure(s, algorithm="gpu-learned")
        sv.initialize()
        t0 = time.perf_counter()
        losses = net.train(sv._fem, steps=steps, lr=lr, seed=100 + j, smooth=smooth, pairs=pairs)
        first, last = float(np.mean(losses[:50])), float(np.mean(losses[-200:]))
        summary.append((seed, first, last))
        if log is not None:
            n = [len(a) for a in s.axes]
            log(f"seed {seed} {n[0]}x{n[1]}x{n[2]}: loss {first:.3f} -> {last:.3f} ({time.perf_counter() - t0:.1f} s)")
        del sv
    return net, summary


def load_c2(path=WEIGHTS_C2):
    """The shipped network trained by :func:`train_c2`."""
    from . import _native

    net = _native.UNet(seed=0)
    net.load(path)
    return net


def time_c2(seed, reps=3):
    """(forward ms, preconditioner application ms) of the shipped network on learned_c2(seed)."""
    from . import structures as S
    from . import thermal as TH

    sv = TH.solver_for_structure(S.learned_c2(seed=seed), algorithm="gpu-learned")
    sv.initialize()
    return load_c2().time_apply(sv._fem, reps=reps)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--time", type=int, default=None, metavar="SEED",
                    help="time the shipped network on learned_c2(SEED) instead of training")
    ap.add_argument("--out", default=str(WEIGHTS_C2))
    ap.add_argument("--steps", type=int, default=STEPS_PER_STRUCTURE, help="pairs per training structure")
    ap.add_argument("--pairs", default="jacobi", choices=["jacobi", "cg"])
    ap.add_argument("--lr", type=float, default=1e-3)
    args = ap.parse_args(argv)
    if args.time is not None:
        fwd, app = time_c2(args.time)
        print(f"forward {1e3 * fwd:.1f} us, preconditioner application {1e3 * app:.1f} us")
        return 0
    smooth = (5, 60) if args.pairs == "jacobi" else (20, 300)
    net, _ = train_c2(steps=args.steps, lr=args.lr, smooth=smooth, pairs=args.pairs)
    out = pathlib.Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    net.save(out)
    print("saved", out)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
