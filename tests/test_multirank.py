"""The benchmark's multi-rank host path on CPU: two gloo ranks (world size 2, rendezvous on
127.0.0.1) share a barrier, a max and a sum, as bench.py does around its timed region
(the solve itself has no collective: every rank runs an independent replica); under
torchrun the reference arm prints from rank 0 only and the other ranks exit 0 without
work."""
import json
import os
import socket
import subprocess
import sys
import pathlib

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    env = dict(os.environ)
    env.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "MASTER_ADDR": "127.0.0.1",
                "MASTER_PORT": str(port)})
    return env


def test_two_gloo_ranks_reduce_max_and_sum():
    port = _free_port()
    code = ("import json, bench\n"
            "d = bench.Dist()\n"
            "d.barrier()\n"
            "out = {'rank': d.rank, 'max': d.max(1.5 + d.rank), 'sum': d.sum(2.0 + d.rank)}\n"
            "d.barrier()\n"
            "d.close()\n"
            "print(json.dumps(out))\n")
    procs = [subprocess.Popen([sys.executable, "-c", code], cwd=ROOT, env=_env(r, 2, port), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in (0, 1)]
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=180)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["max"] == 2.5  # max over ranks of 1.5 + rank
        assert o["sum"] == 5.0  # 2.0 + 3.0


def test_reference_arm_runs_on_rank_0_only():
    port = _free_port()
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=_env(1, 2, port), capture_output=True, text=True, timeout=180)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
