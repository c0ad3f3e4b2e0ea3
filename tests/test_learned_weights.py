"""The shipped network weights of the learned preconditioner (plask_gb300/data/unet_c2.bin,
written by plgpu_unet_save): file layout, parameter count of the architecture, checksum."""
import struct

import numpy as np

from oracle import unet_ref as U
from plask_gb300 import learned as LN


def _fnv1a64(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_shipped_weights_file_is_intact():
    raw = LN.WEIGHTS_C2.read_bytes()
    assert raw[:8] == b"PLGPUNET"
    (version,) = struct.unpack_from("<I", raw, 8)
    (n,) = struct.unpack_from("<Q", raw, 12)
    assert version == 1
    expected = sum(taps * cin * cout for _, cin, cout, taps in U.LAYERS) + U.HEAD
    assert n == expected
    body = raw[20:20 + 4 * n]
    (checksum,) = struct.unpack_from("<Q", raw, 20 + 4 * n)
    assert len(raw) == 20 + 4 * n + 8
    assert checksum == _fnv1a64(body)
    w = np.frombuffer(body, dtype="<f4")
    assert np.all(np.isfinite(w)) and np.any(w != 0.0)


def test_training_recipe_covers_twenty_thousand_pairs():
    assert len(LN.TRAIN_SEEDS) * LN.STEPS_PER_STRUCTURE == 20000
    assert not set(LN.TRAIN_SEEDS) & {2000, 2001, 2002}  # the evaluation structures
