"""Batched solves of a sweep of independent structures (the uneven-size sweep of the
layered generator): concurrent solves give the same temperatures as one-at-a-time
solves, bit for bit at the same grid policy, and the oracle's answer within 1e-6 K;
the autotuner returns a working configuration."""
import numpy as np
import pytest

from oracle import fem3d as O
from plask_gb300 import _native
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

pytestmark = pytest.mark.gpu

TOL_T = 1e-6  # K


def _solvers(structs):
    out = []
    for s in structs:
        sv = TH.solver_for_structure(s, ordering="best", algorithm="gpu-mixed")
        sv.initialize()
        out.append(sv)
    return out


def test_batch_equals_one_at_a_time_and_oracle():
    structs = S.sweep_c3(seed=3300, count=10, lo=20, hi=34)
    seq = _solvers(structs)
    for sv in seq:
        sv.compute()
    bat = _solvers(structs)
    tot, stats, status = _native.batch_compute([sv._fem for sv in bat], loops=0, threads=4)
    assert np.all(status == 0)
    for a, b, st in zip(seq, bat, stats):
        assert np.array_equal(a.temperatures(), b.temperatures())
        assert st["loops"] == a.stats["loops"] and st["inner_iterations"] == a.stats["inner_iterations"]
    for k in (0, 7):
        p = O.from_structure(structs[k], order=bat[k].mesh.ordering)
        To, _, _ = O.compute(p)
        assert np.max(np.abs(bat[k]._full_temperature() - To)) <= TOL_T


def test_batch_tuner_picks_a_configuration_that_solves():
    structs = S.sweep_c3(seed=3200, count=6, lo=20, hi=32)
    svs = _solvers(structs)
    fems = [sv._fem for sv in svs]
    threads, share, timings = _native.batch_tune(fems, loops=0, max_threads=4)
    print("tuned threads", threads, "share", share, "solves/s per trial", timings)
    assert threads in (1, 2, 4) and share in (1, threads)
    assert np.all(timings > 0)
    for f in fems:
        f.invalidate()
    _native.batch_compute(fems, loops=0, threads=threads)
    p = O.from_structure(structs[3], order=svs[3].mesh.ordering)
    To, _, _ = O.compute(p)
    assert np.max(np.abs(svs[3]._full_temperature() - To)) <= TOL_T
