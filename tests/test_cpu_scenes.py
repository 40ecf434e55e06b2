"""Seeded workload generators (host only)."""
import math

import numpy as np

from vkxpbd import scenes


def test_batch_counts_log_uniform_and_seeded():
    a = scenes.batch_counts(512, 1024, 65536, seed=46)
    assert a == scenes.batch_counts(512, 1024, 65536, seed=46)
    assert len(a) == 512 and min(a) >= 1024 and max(a) <= 65536
    # log-uniform: the median sits near the geometric mean 8192
    assert 4096 < np.median(a) < 16384


def test_pile_of_matches_cube_pile():
    a = scenes.pile_of(4096, seed=42).positions
    b = scenes.pile().positions
    assert a.shape == b.shape
    assert np.max(np.abs(a - b)) < 1e-6


def test_pile_of_exact_counts_fill_bottom_up():
    for n in (1, 2, 7, 1000, 1037, 4097):
        p = scenes.pile_of(n, jitter=0.0).positions
        assert p.shape == (n, 3)
        side = max(1, int(math.ceil(round(n ** (1.0 / 3.0), 9))))
        # only the top layer may be partial
        z = np.round((p[:, 2] - 0.02) / 0.02).astype(int)
        full = z < z.max()
        assert np.sum(full) == (z.max()) * side * side


def test_batch_concat_and_offsets():
    batch = scenes.Batch([scenes.pile_of(c, seed=46 + s) for s, c in enumerate([5, 9, 1])])
    assert batch.counts == [5, 9, 1] and batch.n == 15
    x = batch.concat("positions")
    assert x.shape == (15, 3) and x.dtype == np.float32
    assert np.array_equal(x[5:14], batch.scenes[1].positions)
