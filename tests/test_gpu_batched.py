"""Batched scenes (xpbd_batch_init) vs one CPU oracle per scene.

Each scene of a batch has its own hash grid, so its particles must come out
bit-identical to the same scene stepped alone by the oracle (the xpbd_batch_*
contract: batching changes the launch count, never the result).
"""
import numpy as np
import pytest

from helpers import assert_bitexact, config_for, make_pair
import scenes

pytestmark = pytest.mark.gpu


def _batched(batch, cfg):
    import vkxpbd

    g = vkxpbd.XpbdSolver()
    g.init_batched(cfg, batch.counts)
    for sc in batch.scenes[:1]:
        for (v, t, margin, wt) in sc.meshes:
            g.add_mesh(v, t, shape_margin=margin, is_watertight=wt)
    g.finalize_meshes()
    g.set_particles(batch.concat("positions"), batch.concat("velocities"), batch.concat("inv_mass"),
                    batch.concat("radii"), batch.concat("flags"))
    return g


def _compare(g, oracles, off, frames, dt, substeps, iterations, what):
    for f in range(frames):
        g.step(dt, substeps, iterations)
        x, v = g.get_positions(), g.get_velocities()
        for s, orc in enumerate(oracles):
            orc.step(dt, substeps, iterations)
            a, b = off[s], off[s + 1]
            assert_bitexact(x[a:b], orc.get_positions(), f"{what} scene {s} positions frame {f}")
            assert_bitexact(v[a:b], orc.get_velocities(), f"{what} scene {s} velocities frame {f}")


def test_batched_uneven_piles_bitexact():
    counts = [700, 1, 2048, 64, 1500, 333]
    batch = scenes.Batch([scenes.pile_of(c, seed=46 + s, name=f"p{s}") for s, c in enumerate(counts)])
    cfg = config_for(batch)
    g = _batched(batch, cfg)
    assert g.scene_count() == len(counts)
    off = g.scene_offsets()
    assert list(off) == [0] + list(np.cumsum(counts))
    oracles = [make_pair(sc, cfg, gpu=False)[1] for sc in batch.scenes]
    _compare(g, oracles, off, 6, 1.0 / 60.0, 10, 1, "batched piles")


def test_batched_sorted_keys_per_scene():
    """Keys are (scene << 21) | cell; within a scene the order is the scene's own sort."""
    counts = [300, 900, 5]
    batch = scenes.Batch([scenes.pile_of(c, seed=46 + s) for s, c in enumerate(counts)])
    cfg = config_for(batch)
    g = _batched(batch, cfg)
    oracles = [make_pair(sc, cfg, gpu=False)[1] for sc in batch.scenes]
    g.step(1.0 / 60.0, 1, 1)
    keys, ids = g.get_sorted_cells(), g.get_sorted_point_ids()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    off = g.scene_offsets()
    for s, orc in enumerate(oracles):
        orc.step(1.0 / 60.0, 1, 1)
        oc, oi = orc.get_sorted()
        a, b = off[s], off[s + 1]
        assert np.all(keys[a:b] >> 21 == s)
        assert_bitexact(keys[a:b] & ((1 << 21) - 1), oc, f"scene {s} cells")
        assert_bitexact(ids[a:b] - a, oi, f"scene {s} ids")


def test_batched_mesh_scenes_bitexact():
    """Scenes sharing a heightfield mesh: mesh contacts per scene, plus iterations > 1."""
    hv, ht = scenes.heightfield(32, extent=0.4, amplitude=0.02)
    batch = []
    for s, c in enumerate([1000, 3000, 250]):
        sc = scenes.pile_of(c, spacing=0.01, radius=0.005, jitter=0.001, bottom_z=0.06, seed=46 + s)
        sc.meshes.append((hv, ht, 0.0, None))
        batch.append(sc)
    batch = scenes.Batch(batch)
    cfg = config_for(batch)
    g = _batched(batch, cfg)
    oracles = [make_pair(sc, cfg, gpu=False)[1] for sc in batch.scenes]
    _compare(g, oracles, g.scene_offsets(), 5, 1.0 / 60.0, 5, 2, "batched mesh")


def test_batched_many_scenes_4_passes():
    """More than 8 scenes: the key grows past 24 bits and the sort takes a fourth pass."""
    counts = scenes.batch_counts(300, 16, 200, seed=46)
    batch = scenes.Batch([scenes.pile_of(c, seed=46 + s) for s, c in enumerate(counts)])
    cfg = config_for(batch)
    g = _batched(batch, cfg)
    tuned = g.autotune()  # any sort variant must give the same result (stable sort)
    assert tuned["bits"] in (7, 8) and len(tuned["sort_us"]) == 8
    rng = np.random.default_rng(0)
    pick = sorted(rng.choice(len(counts), 6, replace=False).tolist())
    oracles = {s: make_pair(batch.scenes[s], cfg, gpu=False)[1] for s in pick}
    off = g.scene_offsets()
    for f in range(4):
        g.step(1.0 / 60.0, 10, 1)
        x = g.get_positions()
        for s, orc in oracles.items():
            orc.step(1.0 / 60.0, 10, 1)
            assert_bitexact(x[off[s]:off[s + 1]], orc.get_positions(), f"scene {s} frame {f}")


@pytest.mark.parametrize("bits,items", [(8, 2), (8, 4), (8, 8), (8, 16), (7, 4), (7, 8), (7, 16), (7, 32)])
def test_every_sort_variant_bitexact(bits, items):
    """Each onesweep variant the autotuner chooses from gives the same (stable) result."""
    from helpers import small_pile

    sc = small_pile(12)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.set_sort_variant(bits, items)
    for f in range(3):
        g.step(1.0 / 60.0, 10, 1)
        orc.step(1.0 / 60.0, 10, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"frame {f}")


def test_batched_scenes_with_boxes_bitexact():
    """Uneven piles with 0-3 dynamic boxes each in one batched solver (bodies assigned to
    their scenes): every scene's particles and boxes equal that scene stepped alone."""
    full = scenes.batched_piles_with_boxes(n_scenes=4, lo=150, hi=900, max_boxes=3, seed=52)
    batch = scenes.Batch(full.scenes)
    cfg = config_for(batch)
    import vkxpbd

    g = vkxpbd.XpbdSolver()
    g.init_batched(cfg, batch.counts)
    meshes, bodies, body_scene = scenes.batch_bodies(batch)
    for (v, t, margin, wt) in meshes:
        g.add_mesh(v, t, shape_margin=margin, is_watertight=wt)
    g.finalize_meshes()
    g.set_bodies(bodies.q, bodies.qd, bodies.com, bodies.inertia, bodies.inv_inertia, bodies.inv_mass,
                 bodies.flags)
    g.set_body_scenes(body_scene)
    g.set_particles(batch.concat("positions"), batch.concat("velocities"), batch.concat("inv_mass"),
                    batch.concat("radii"), batch.concat("flags"))
    assert sum(len(sc.meshes) - 1 for sc in batch.scenes) > 0, "the seed must give some boxes"
    oracles = [make_pair(sc, cfg, gpu=False)[1] for sc in batch.scenes]
    off = g.scene_offsets()
    for f in range(30):
        g.step(1.0 / 60.0, 10, 1)
        x, q = g.get_positions(), g.get_body_q()
        for s, orc in enumerate(oracles):
            orc.step(1.0 / 60.0, 10, 1)
            assert_bitexact(x[off[s]:off[s + 1]], orc.get_positions(), f"scene {s} positions frame {f}")
            assert_bitexact(q[body_scene == s], orc.get_body_q()[1:], f"scene {s} boxes frame {f}")
