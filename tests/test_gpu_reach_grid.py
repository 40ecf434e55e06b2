"""Contact generation with the per-mesh reach grids vs the CPU oracle (which has none).

The grids let the collision kernel skip the BVH traversal of a particle that cannot
reach any leaf of a mesh; the skipped query must end exactly as the traversal would
(no contact). These cases put many particles right around the reach boundary, with
mixed radii, several meshes (open heightfield, watertight box, shape margins),
non-finite particles, and changes that must rebuild the grids (radii, contact
margin, moved mesh vertices). Bar: bit-exact contacts and states.
"""
import numpy as np
import pytest

from helpers import assert_bitexact, config_for, make_pair
import scenes

pytestmark = pytest.mark.gpu


def _band_scene(n=20000, seed=7, r_lo=0.001, r_hi=0.02):
    """Particles at heights around the heightfield surface and around a box, with the
    offsets concentrated near margin + radius (the reach boundary)."""
    rng = np.random.default_rng(seed)
    hv, ht = scenes.heightfield(48, extent=0.5, amplitude=0.03)
    bv, bt = scenes.box_mesh((0.06, 0.05, 0.04), center=(0.1, -0.05, 0.12),
                             quat_xyzw=(0.0, 0.0, 0.3826834, 0.9238795))
    radii = rng.uniform(r_lo, r_hi, n).astype(np.float32)
    # points on random heightfield triangles, lifted by an offset around the reach
    tri = rng.integers(0, ht.shape[0], n)
    b = rng.random((n, 2))
    flip = b.sum(1) > 1.0
    b[flip] = 1.0 - b[flip]
    a_, b_, c_ = hv[ht[tri, 0]], hv[ht[tri, 1]], hv[ht[tri, 2]]
    surf = a_ + b[:, :1] * (b_ - a_) + b[:, 1:] * (c_ - a_)
    reach = 0.01 + radii
    off = reach * rng.choice([-1.0, 1.0], n) * (1.0 + rng.normal(0.0, 0.05, n))
    off[: n // 4] = rng.uniform(-0.08, 0.08, n // 4)
    pos = surf.copy()
    pos[:, 2] += off
    # a quarter around the box: random directions from its centre, at distances around its size
    k = n // 4
    d = rng.normal(size=(k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos[-k:] = np.array([0.1, -0.05, 0.12]) + d * rng.uniform(0.03, 0.12, (k, 1))
    sc = scenes.pile(dims=(1, 1, 1), radius=0.01)
    sc.positions = pos.astype(np.float32)
    sc.velocities = np.zeros_like(sc.positions)
    sc.inv_mass = np.full(n, 1000.0, np.float32)
    sc.radii = radii
    sc.flags = np.ones(n, np.int32)
    sc.meshes = [(hv, ht, 0.0, None), (bv, bt, 0.004, None)]
    return sc


def _contacts_equal(g, orc, what):
    g.collide_only()
    orc.collide_only()
    assert g.last_contact_count == orc.last_contact_count, what
    c = orc.get_contacts()
    assert_bitexact(g.get_contact_particles(), c["particles"], f"{what} particles")
    assert_bitexact(g.get_contact_shapes(), c["shapes"], f"{what} shapes")
    assert_bitexact(g.get_contact_normals(), c["normals"], f"{what} normals")
    assert_bitexact(g.get_contact_body_positions(), c["body_positions"], f"{what} body positions")
    return g.last_contact_count


def test_reach_band_contacts_bitexact():
    sc = _band_scene()
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg, max_contacts=3 * sc.n)
    count = _contacts_equal(g, orc, "band")
    assert 0 < count < 2 * sc.n
    for f in range(3):
        g.step(1.0 / 60.0, 5, 1)
        orc.step(1.0 / 60.0, 5, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"band positions frame {f}")


def test_reach_grid_rebuilds_on_radius_margin_and_mesh_changes():
    sc = _band_scene(n=8000, seed=11, r_lo=0.002, r_hi=0.006)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg, max_contacts=3 * sc.n)
    _contacts_equal(g, orc, "initial")
    # larger radii: the reach grows
    big = (sc.radii * 3.0).astype(np.float32)
    for s in (g, orc):
        s.set_particles(sc.positions, sc.velocities, sc.inv_mass, big, sc.flags)
    _contacts_equal(g, orc, "radii x3")
    # a wider contact margin (a fresh oracle with the new configuration, same state)
    cfg.soft_contact_margin = 0.03
    g.update_config(cfg)
    sc.radii = big
    _, orc = make_pair(sc, cfg, max_contacts=3 * sc.n, gpu=False)
    _contacts_equal(g, orc, "margin 0.03")
    # the heightfield moved and rescaled: its grid covers a new box
    hv = sc.meshes[0][0].copy()
    hv[:, :2] *= 1.3
    hv[:, 2] += 0.05
    g.update_mesh(0, hv, None)
    orc.update_mesh(0, hv, None)
    _contacts_equal(g, orc, "moved mesh")


def test_reach_grid_non_finite_particles_bitexact():
    sc = _band_scene(n=2000, seed=5)
    sc.positions[0] = [np.nan, 0.0, 0.0]
    sc.positions[1] = [np.inf, 0.0, 0.0]
    sc.positions[2] = [0.0, 0.0, -np.inf]
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg, max_contacts=3 * sc.n)
    _contacts_equal(g, orc, "non-finite positions")
    # a radius of +inf reaches every mesh from anywhere: the grids are left out
    r = sc.radii.copy()
    r[3] = np.inf
    for s in (g, orc):
        s.set_particles(np.nan_to_num(sc.positions, nan=0.0, posinf=1.0, neginf=-1.0), None, sc.inv_mass, r,
                        sc.flags)
    _contacts_equal(g, orc, "infinite radius")
