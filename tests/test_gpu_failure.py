"""Failure detection without a GPU fault: the sort's bounded look-back wait.

The reference waits on its fence with no timeout (src/scene.cpp:1003), and its radix sort has
no cross-workgroup wait at all. Here the onesweep pass's decoupled look-back spins on its
predecessors' published prefixes, bounded by a timer. xpbd_debug_lookback_hold makes one tile
of the first radix pass never publish, so the wait of the tile after it runs out (1 ms here),
the kernel records the time-out in the status word and returns, and the host raises. No trap,
no fault, no unbounded wait: the context stays usable and the next normal step is bit-exact.
"""
import numpy as np
import pytest

import scenes
from helpers import assert_bitexact, config_for, make_pair

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def test_lookback_timeout_raises_and_the_next_step_is_exact():
    import vkxpbd

    # 13,824 particles, 21-bit keys: three radix passes of seven 2,048-key tiles
    sc = scenes.pile(dims=(24, 24, 24))
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.step(DT, 2, 1)
    orc.step(DT, 2, 1)
    assert_bitexact(g.get_positions(), orc.get_positions(), "before the hold")
    vkxpbd.debug_lookback_hold(1, 1_000_000)  # tile 1 never publishes; waits give up after 1 ms
    try:
        with pytest.raises(RuntimeError, match="timed out in the onesweep look-back"):
            g.step(DT, 2, 1)
        error_bits, lookback_timeouts, _, _ = g.get_status()
        assert error_bits & 1, error_bits
        assert lookback_timeouts >= 1, lookback_timeouts
    finally:
        vkxpbd.debug_lookback_hold(-1)
    # the held frame's result is discarded: restart both from the oracle's state
    g.set_particles(orc.get_positions(), orc.get_velocities())
    for f in range(3):
        g.step(DT, 2, 1)
        orc.step(DT, 2, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"after the hold, frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"after the hold, frame {f}")
    assert g.get_status()[0] == 0
    assert np.isfinite(g.get_positions()).all()


def test_debug_hold_rejects_bad_limits():
    import vkxpbd

    with pytest.raises(RuntimeError, match="wait limit"):
        vkxpbd.debug_lookback_hold(0, 0)
    with pytest.raises(RuntimeError, match="wait limit"):
        vkxpbd.debug_lookback_hold(0, 2_000_000_000)
    vkxpbd.debug_lookback_hold(-1)
