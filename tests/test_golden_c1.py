"""The 128x128x200 reference fixture (the reference's NSPCG at zeta 1e-12, written by
tests/golden/make_golden_c1.py) on the CPU: the generator still gives the inputs the answers
belong to, and the stored answers are consistent with each other.  The GPU comparison is in
tests/test_gpu_parity_full.py."""
import json
import pathlib
import sys

import numpy as np
import pytest

from plask_gb300 import structures as S

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
FIX = HERE / "golden" / "static3d_layered_c1_128x128x200_nspcg.npz"

pytestmark = pytest.mark.skipif(not FIX.exists(), reason="fixture not generated")


def _load():
    d = np.load(FIX)
    return json.loads(str(d["meta"])), d


def test_generator_still_gives_the_fixture_inputs():
    from make_golden_c1 import inputs_match

    meta, _ = _load()
    assert inputs_match(S.layered_c1(), meta["inputs"])


def test_stored_answers_are_consistent():
    meta, d = _load()
    k, j, i = meta["hot_node"]
    assert d["plane"].shape == (128, 128) and d["line"].shape == (200,)
    assert d["plane"][j, i] == meta["max_t"] == d["line"][k]
    assert np.max(d["plane"]) == meta["max_t"] and np.max(d["line"]) == meta["max_t"]
    assert np.all(d["T_idx"] <= meta["max_t"]) and np.all(d["T_idx"] >= 300.0 - 1e-9)
    loops = meta["loops"]
    assert len(loops) == 5 and loops[-1]["err"] <= 0.05 < loops[-2]["err"]
    assert abs(loops[-1]["maxT"] - meta["max_t"]) < 1e-12
    assert meta["rel_residual"] < 1e-14
    # the bottom plane carries the Dirichlet 300 K
    assert d["line"][0] == 300.0
