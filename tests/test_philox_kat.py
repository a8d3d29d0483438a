"""Pin the numpy Philox4x32-10 used to check the GPU Langevin noise against
the published known-answer vectors of the algorithm (Random123 kat_vectors,
philox4x32_10 entries).  CPU only."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from philox_ref import philox4x32_10, stoch_noise  # noqa: E402

KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_philox_known_answers():
    for ctr, key, want in KAT:
        got = philox4x32_10(tuple(np.array([c], dtype=np.uint64) for c in ctr), key)
        assert tuple(int(g[0]) for g in got) == want


def test_noise_statistics():
    g = stoch_noise(12345, 7, 200000)
    assert abs(g.mean()) < 5e-3 and abs(g.var() - 1.0) < 1e-2
