"""Frame cache (xpbd_record_start / xpbd_record_stop): the .npy files written by
the writer thread equal get_positions() after each step, as the add-on's
np.save(frame_%04d.npy, solver.get_positions()) loop (newton_vulkan_plugin.py:626-631)."""
import os

import numpy as np
import pytest

from helpers import config_for, make_pair, small_pile

pytestmark = pytest.mark.gpu


def test_recorded_frames_equal_positions(tmp_path):
    sc = small_pile(8)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.record_start(str(tmp_path), first_frame=1)
    for f in range(5):
        g.step_async(1.0 / 60.0, 10, 1)  # queued: the copy and the file write overlap the next frame
    n = g.record_stop()
    assert n == 5
    for f in range(1, 6):
        orc.step(1.0 / 60.0, 10, 1)
        a = np.load(os.path.join(tmp_path, f"frame_{f:04d}.npy"))
        assert a.dtype == np.float32 and a.shape == (sc.n, 3)
        assert np.array_equal(a.view(np.uint32), orc.get_positions().view(np.uint32)), f
    # stepping after the stop writes nothing more
    g.step(1.0 / 60.0, 10, 1)
    assert not os.path.exists(os.path.join(tmp_path, "frame_0006.npy"))


def test_record_to_missing_directory_reports_error(tmp_path):
    sc = small_pile(4)
    g, _ = make_pair(sc, config_for(sc))
    g.record_start(str(tmp_path / "does_not_exist"), first_frame=1)
    g.step(1.0 / 60.0, 2, 1)
    with pytest.raises(RuntimeError):
        g.record_stop()
