"""Hash-grid aliasing: particles 128 cells apart share the reference's 21-bit cell key.

One-scene solvers of 32,768 particles or more (or with VKXPBD_SPLIT_KEYS set, as here) sort
split keys (the reference's key plus bit 7 of each axis' unwrapped cell coordinate) so that
the neighbour loop skips particles 128 cells away, which the reference visits and rejects by
distance. These scenes put clusters exactly 128 and 256
cells apart along x, y and z, one cluster across the 128-cell boundary and one at negative
coordinates, so that wrapped cells hold several clusters. Bar: bit-exact states, contacts and
the sorted-order getters (which report the reference's 21-bit layout) against the oracle.
"""
import numpy as np
import pytest

from helpers import assert_bitexact, config_for, make_pair
import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _split_keys(monkeypatch):
    # these scenes are below the particle count from which solvers sort split keys by
    # themselves; the variable makes them sort split keys too
    monkeypatch.setenv("VKXPBD_SPLIT_KEYS", "1")


def _alias_scene(seed=21, n_side=7):
    base = scenes.pile(dims=(n_side, n_side, n_side), spacing=0.02, radius=0.01, jitter=0.002, bottom_z=0.02,
                       seed=seed)
    cell = 0.02  # search radius 2 r
    period = 128 * cell
    shifts = [
        (0.0, 0.0, 0.0),
        (period, 0.0, 0.0),          # same wrapped cells, other alias bit in x
        (2 * period, 0.0, 0.0),      # same split keys too (256 cells)
        (0.0, period, 0.0),
        (0.0, 0.0, period),          # falls from 2.56 m
        (period - 0.07, 0.5, 0.0),   # across the 128-cell boundary in x
        (-period - 0.03, -0.4, 0.0),  # negative coordinates
    ]
    rng = np.random.default_rng(seed)
    pos = []
    for s in shifts:
        p = base.positions.astype(np.float64) + np.asarray(s)
        p[:, :2] += rng.uniform(-0.003, 0.003, size=(p.shape[0], 2))
        pos.append(p)
    x = np.concatenate(pos).astype(np.float32)
    n = x.shape[0]
    sc = scenes.pile(dims=(1, 1, 1))
    sc.positions = x
    sc.velocities = rng.normal(0.0, 0.2, size=(n, 3)).astype(np.float32)
    sc.inv_mass = np.full(n, 1000.0, np.float32)
    sc.radii = np.full(n, 0.01, np.float32)
    sc.flags = np.ones(n, np.int32)
    return sc


def _check_grid(g, orc, what):
    oc, oi = orc.get_sorted()
    assert_bitexact(g.get_sorted_cells(), oc, f"{what} sorted cells")
    assert_bitexact(g.get_sorted_point_ids(), oi, f"{what} sorted ids")
    assert_bitexact(g.get_cell_starts(), orc.get_cell_starts(), f"{what} cell starts")
    assert_bitexact(g.get_cell_ends(), orc.get_cell_ends(), f"{what} cell ends")


def test_aliased_clusters_bitexact():
    sc = _alias_scene()
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    for f in range(8):
        g.step(1.0 / 60.0, 4, 1)
        orc.step(1.0 / 60.0, 4, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"velocities frame {f}")
        assert g.last_contact_count == orc.last_contact_count, f"contact count frame {f}"
        if f in (0, 7):
            _check_grid(g, orc, f"frame {f}")
    # the wrapped cells really are shared: several clusters per 21-bit key
    cells = g.get_sorted_cells().astype(np.int64)
    assert cells.max() < (1 << 21)
    _, counts = np.unique(cells, return_counts=True)
    assert counts.max() >= 4


def test_aliased_clusters_two_iterations_with_cohesion():
    sc = _alias_scene(seed=5, n_side=6)
    cfg = config_for(sc, particle_cohesion=0.004, particle_adhesion=0.01)
    g, orc = make_pair(sc, cfg)
    for f in range(4):
        g.step(1.0 / 60.0, 3, 2)
        orc.step(1.0 / 60.0, 3, 2)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"velocities frame {f}")
    _check_grid(g, orc, "cohesion")


def test_far_and_clamped_coordinates_bitexact():
    """Particles beyond 2^20 cells clamp to cell 0 on each axis (grid_cell_indices.comp:21-23)
    under both keys; far particles share wrapped cells with the pile near the origin."""
    sc = _alias_scene(seed=9, n_side=5)
    rng = np.random.default_rng(9)
    far = np.array([[-3.0e4, 0.0, 0.5], [-3.0e4, 0.005, 0.5], [2.0e4, -2.0e4, 1.0], [5.12, 5.12, 5.12],
                    [-5.12, 0.01, 0.3], [1.0e5, 1.0e5, 1.0e5]], np.float32)
    far = np.concatenate([far, far + rng.uniform(-0.004, 0.004, far.shape).astype(np.float32)])
    n0 = sc.n
    sc.positions = np.concatenate([sc.positions, far]).astype(np.float32)
    k = far.shape[0]
    sc.velocities = np.concatenate([sc.velocities, np.zeros((k, 3), np.float32)])
    sc.inv_mass = np.concatenate([sc.inv_mass, np.full(k, 1000.0, np.float32)])
    sc.radii = np.concatenate([sc.radii, np.full(k, 0.01, np.float32)])
    sc.flags = np.concatenate([sc.flags, np.ones(k, np.int32)])
    assert sc.n == n0 + k
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    for f in range(4):
        g.step(1.0 / 60.0, 4, 1)
        orc.step(1.0 / 60.0, 4, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"velocities frame {f}")
    _check_grid(g, orc, "far")
