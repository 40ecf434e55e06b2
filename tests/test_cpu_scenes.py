"""Seeded workload generators (host only)."""
import math

import numpy as np

import scenes


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


def test_oracle_config_has_the_reference_defaults():
    """The oracle's own SolverConfig (used where no product code may load) carries the same
    defaults as vkxpbd.SolverConfig (src/scene.h:15-40)."""
    import oracle as O
    import vkxpbd

    a, b = O.SolverConfig(), vkxpbd.SolverConfig()
    for k, va in vars(a).items():
        vb = getattr(b, k)
        if k == "gravity":
            assert np.allclose(list(vb), va, rtol=1e-6), k
        elif isinstance(va, bool):
            assert bool(vb) == va, k
        else:
            assert abs(float(vb) - float(va)) <= 1e-6 * max(1.0, abs(float(va))), k


def test_reference_arm_path_loads_no_product_code():
    """The benchmark's reference arm builds its scene and configuration and steps the oracle
    without importing vkxpbd or loading libxpbd_gb300.so."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys, os\n"
        f"sys.path[:0] = [{os.path.join(root, 'newton-xpbd-vulkan_gb300')!r}, {os.path.join(root, 'oracle')!r}, "
        f"{os.path.join(root, 'tests')!r}]\n"
        "import scenes\n"
        "from helpers import config_for, make_pair\n"
        "sc = scenes.pile(dims=(6, 6, 6))\n"
        "cfg = config_for(sc, gpu=False)\n"
        "_, orc = make_pair(sc, cfg, gpu=False)\n"
        "orc.step(1.0 / 60.0, 1, 1)\n"
        "assert 'vkxpbd' not in sys.modules, 'vkxpbd imported'\n"
        "maps = open('/proc/self/maps').read() if os.path.exists('/proc/self/maps') else ''\n"
        "assert 'libxpbd_gb300' not in maps, 'product library loaded'\n"
        "print('ok')\n"
    )
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stderr
