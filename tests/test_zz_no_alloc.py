"""plgpu_fem3d_mult_noalloc: A x without any device allocation during the call.

It exists for callers that cannot allocate device memory when they need the
product -- a framework that has reserved the whole GPU for its own allocator, or
a latency-critical loop that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree.  Its staging buffer is a static device array of 2,097,152
doubles shared by all calls, whose address is looked up when a handle is created.
These tests call it through the C ABI and compare it with plgpu_fem3d_mult on the
same inputs, two calls in a row, on 3D and planar handles, and check in a fresh
process (CUDA's default lazy module loading) that repeated calls leave the
device's free memory unchanged.  This file is collected last so that a failure
here stops a -x run only after every other test.
"""
import os
import pathlib
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from plask_gb300 import _native
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH
from plask_gb300 import thermal2d as T2

ROOT = pathlib.Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.gpu

NOALLOC_MAX_NODES = 1 << 21
RTOL64 = 1e-12  # as the operator tests
RTOL32 = 2e-5


def _solver(seed, n, order):
    s = S.layered_c1(seed=seed, n=n)
    s.heatflux = [("left", -1e4)]
    sv = TH.solver_for_structure(s, ordering=order, algorithm="gpu-mixed")
    sv.compute(1)  # sets the handle up on the device and gives a non-uniform temperature
    return sv


@pytest.mark.parametrize("precision,rtol", [(64, RTOL64), (32, RTOL32)])
def test_noalloc_matches_mult_twice_in_a_row(precision, rtol):
    sv = _solver(31, (23, 19, 26), "201")
    fem = sv._fem
    nn, _ = fem.sizes()
    rng = np.random.default_rng(3)
    for _ in range(2):
        x = rng.standard_normal(nn)
        ref = fem.mult(x, precision)
        got = fem.mult_noalloc(x, precision)
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= rtol * scale
        again = fem.mult_noalloc(x, precision)  # the shared array keeps the last call's contents
        assert np.max(np.abs(again - ref)) <= rtol * scale


def test_noalloc_two_handles_in_turn():
    a = _solver(32, (17, 21, 15), "012")
    b = _solver(33, (25, 14, 19), "210")
    rng = np.random.default_rng(4)
    for sv in (a, b, a):
        nn, _ = sv._fem.sizes()
        x = rng.standard_normal(nn)
        ref = sv._fem.mult(x, 64)
        got = sv._fem.mult_noalloc(x, 64)
        assert np.max(np.abs(got - ref)) <= RTOL64 * np.max(np.abs(ref))


def test_noalloc_rejects_meshes_above_the_limit_and_unprepared_handles():
    n = 129  # 129^3 = 2,146,689 nodes > 2,097,152
    assert n ** 3 > NOALLOC_MAX_NODES
    axes = [np.linspace(0.0, 10.0, n)] * 3
    fem = _native.Fem3D(axes, "012")
    try:
        with pytest.raises(_native.BadInput, match="2097152"):
            fem.mult_noalloc(np.zeros(n ** 3), 64)
    finally:
        fem.close()
    small = _native.Fem3D([np.linspace(0.0, 1.0, 5)] * 3, "012")
    try:
        with pytest.raises(_native.NativeError, match="set up"):
            small.mult_noalloc(np.zeros(125), 64)
    finally:
        small.close()


@pytest.mark.parametrize("cls", [T2.Static2D, T2.StaticCyl])
def test_noalloc_on_planar_handles(cls):
    s = S.layered_2d(seed=71, n=(25, 31), anisotropic=True)
    s.convection = [("top", 3e3, 300.0)]
    sv = T2.solver_for_structure2d(s, cls=cls, ordering="10")
    sv.compute(1)
    fem = sv._fem
    nn, _ = fem.sizes()
    rng = np.random.default_rng(6)
    for precision, rtol in ((64, RTOL64), (32, RTOL32)):
        for _ in range(2):
            x = 300.0 + rng.standard_normal(nn)
            ref = fem.mult(x, precision)
            got = fem.mult_noalloc(x, precision)
            assert np.max(np.abs(got - ref)) <= rtol * np.max(np.abs(ref))


_FREE_MEMORY_PROBE = textwrap.dedent("""
    import sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    from plask_gb300 import structures as S
    from plask_gb300 import thermal as TH
    s = S.layered_c1(seed=34, n=(21, 18, 24))
    sv = TH.solver_for_structure(s, ordering="201", algorithm="gpu-mixed")
    sv.compute(1)
    fem = sv._fem
    nn, _ = fem.sizes()
    x = np.random.default_rng(7).standard_normal(nn)
    ref = fem.mult(x, 64)
    fem.mult_noalloc(x, 64)   # warm-up: the kernels of the multiply are loaded by now
    fem.mult_noalloc(x, 32)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(5):
        y64 = fem.mult_noalloc(x, 64)
        y32 = fem.mult_noalloc(x, 32)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info(0)[0]
    err = float(np.max(np.abs(y64 - ref)) / np.max(np.abs(ref)))
    print("FREE", free0, free1, "ERR", err)
""")


def test_noalloc_leaves_free_memory_unchanged_in_a_fresh_process():
    pytest.importorskip("torch")
    env = dict(os.environ)
    env.pop("CUDA_MODULE_LOADING", None)  # the driver's default: lazy loading
    r = subprocess.run([sys.executable, "-c", _FREE_MEMORY_PROBE, str(ROOT)], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1].split()
    free0, free1, err = int(line[1]), int(line[2]), float(line[4])
    assert free1 == free0, f"free device memory changed across no-allocation calls: {free0} -> {free1}"
    assert err <= RTOL64
