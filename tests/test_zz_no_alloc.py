"""plgpu_fem3d_mult_noalloc: A x without any device allocation during the call.

It exists for callers that cannot allocate device memory when they need the
product -- a framework that has reserved the whole GPU for its own allocator, or
a latency-critical loop that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree.  Its staging buffer is a static device array of 2,097,152
doubles shared by all calls.  These tests call it through the C ABI and compare
it with plgpu_fem3d_mult on the same inputs, two calls in a row; this file is
collected last so that a failure here stops a -x run only after every other test.
"""
import numpy as np
import pytest

from plask_gb300 import _native
from plask_gb300 import structures as S
from plask_gb300 import thermal as TH

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
