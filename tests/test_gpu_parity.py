"""CUDA path vs the CPU oracle, through the public vkxpbd API (C ABI underneath).

Bar: bit-exact (uint32 views of float32) for positions, velocities, contacts,
sorted cells/ids and cell tables; the kernels restate the shader arithmetic
operation by operation, so no tolerance is needed. (The reference's own
stated tolerance, 1e-5 relative per substep, is kept in test_tolerance_floor
as the floor these results must also satisfy.)
"""
import numpy as np
import pytest

from helpers import assert_bitexact, config_for, make_pair, mesh_pile, small_pile

pytestmark = pytest.mark.gpu


def _step_compare(g, orc, frames, dt, substeps, iterations, what):
    for f in range(frames):
        g.step(dt, substeps, iterations)
        orc.step(dt, substeps, iterations)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"{what} positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"{what} velocities frame {f}")
        assert g.last_contact_count == orc.last_contact_count, f"{what} contact count frame {f}"


def test_grid_intermediates_bitexact():
    sc = small_pile(12)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.step(1.0 / 60.0, 1, 1)
    orc.step(1.0 / 60.0, 1, 1)
    oc, oi = orc.get_sorted()
    assert_bitexact(g.get_sorted_cells(), oc, "sorted cells")
    assert_bitexact(g.get_sorted_point_ids(), oi, "sorted ids")
    assert_bitexact(g.get_cell_starts(), orc.get_cell_starts(), "cell starts")
    assert_bitexact(g.get_cell_ends(), orc.get_cell_ends(), "cell ends")
    assert np.all(np.diff(g.get_sorted_cells().astype(np.int64)) >= 0)


def test_pile_config1_bitexact():
    """The 4,096-particle pile (plane, particle-particle, restitution 0.2), 10 substeps x 1 iteration."""
    import scenes

    sc = scenes.pile()
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    _step_compare(g, orc, 12, 1.0 / 60.0, 10, 1, "pile")
    c_g, c_o = g.get_contact_particles(), orc.get_contacts()
    assert_bitexact(c_g, c_o["particles"], "contact particles")
    assert_bitexact(g.get_contact_normals(), c_o["normals"], "contact normals")
    assert_bitexact(g.get_contact_body_positions(), c_o["body_positions"], "contact body positions")


@pytest.mark.parametrize("iterations", [2, 3])
def test_pile_multi_iteration_bitexact(iterations):
    sc = small_pile(10)
    cfg = config_for(sc, enable_restitution=False)
    g, orc = make_pair(sc, cfg)
    _step_compare(g, orc, 6, 1.0 / 60.0, 4, iterations, f"iters={iterations}")


def test_cohesion_adhesion_flags_bitexact():
    sc = small_pile(10)
    n = sc.n
    flags = np.ones(n, np.int32)
    flags[::7] = 0          # inactive
    flags[3::11] = 3        # active + proxy
    sc.flags = flags
    sc.inv_mass[::13] = 0.0  # some kinematic particles
    cfg = config_for(sc, particle_cohesion=0.002, particle_adhesion=0.001, soft_contact_restitution=0.5)
    g, orc = make_pair(sc, cfg)
    _step_compare(g, orc, 6, 1.0 / 60.0, 5, 2, "flags")


def test_mesh_heightfield_bitexact():
    sc = mesh_pile(16, 32)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    _step_compare(g, orc, 15, 1.0 / 60.0, 10, 1, "heightfield")
    assert g.last_contact_count > 0
    c = orc.get_contacts()
    for name, key in (("particles", "particles"), ("shapes", "shapes")):
        assert_bitexact(getattr(g, f"get_contact_{name}")(), c[key], f"contact {name}")
    assert_bitexact(g.get_contact_normals(), c["normals"], "contact normals")
    assert_bitexact(g.get_contact_body_positions(), c["body_positions"], "contact body positions")
    assert_bitexact(g.get_contact_body_velocities(), c["body_velocities"], "contact body velocities")


def test_watertight_box_bitexact():
    import scenes

    sc = small_pile(8, spacing=0.02, radius=0.01, bottom_z=0.05)
    bv, bt = scenes.box_mesh((0.05, 0.05, 0.03), center=(0.0, 0.0, 0.03), quat_xyzw=(0.0, 0.0, 0.3826834, 0.9238795))
    sc.meshes.append((bv, bt, 0.002, None))
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    _step_compare(g, orc, 10, 1.0 / 60.0, 5, 1, "box")


def test_collide_only_contacts_bitexact():
    sc = mesh_pile(12, 24)
    sc.positions[:, 2] -= 0.1  # start in contact
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.collide_only()
    orc.collide_only()
    assert g.last_contact_count == orc.last_contact_count > 0
    c = orc.get_contacts()
    assert_bitexact(g.get_contact_particles(), c["particles"], "particles")
    assert_bitexact(g.get_contact_shapes(), c["shapes"], "shapes")
    assert_bitexact(g.get_contact_normals(), c["normals"], "normals")


def test_contact_max_cap_bitexact():
    sc = mesh_pile(12, 24)
    sc.positions[:, 2] -= 0.1
    cfg = config_for(sc)
    cap = 300
    g, orc = make_pair(sc, cfg, max_contacts=cap)
    g.collide_only()
    orc.collide_only()
    assert g.last_contact_count == orc.last_contact_count == cap
    assert_bitexact(g.get_contact_particles(), orc.get_contacts()["particles"], "capped particles")
    _step_compare(g, orc, 4, 1.0 / 60.0, 5, 1, "capped")


def test_contact_max_cap_crossed_during_run_bitexact():
    """A pile falling onto the heightfield: early substeps stay under the cap (every contact
    kept, the rank scan skipped on the device), later ones exceed it (contacts past the cap
    dropped in the canonical order)."""
    sc = mesh_pile(12, 24)
    cfg = config_for(sc)
    cap = 400
    g, orc = make_pair(sc, cfg, max_contacts=cap)
    counts = []
    for f in range(10):
        g.step(1.0 / 60.0, 5, 1)
        orc.step(1.0 / 60.0, 5, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"velocities frame {f}")
        assert g.last_contact_count == orc.last_contact_count, f"contact count frame {f}"
        counts.append(g.last_contact_count)
    assert min(counts) < cap and max(counts) == cap, counts


def test_step_solve_only_bitexact():
    sc = small_pile(8)
    sc.positions[:, 2] -= 0.05
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    orc.collide_only()
    c = orc.get_contacts()
    k = len(c["particles"])
    assert k > 0
    # inject the oracle's contacts in reverse order (multi-contact particles keep their given order)
    p, s, bp, nn = c["particles"][::-1], c["shapes"][::-1], c["body_positions"][::-1], c["normals"][::-1]
    g.set_contact_data(p, s, bp, nn, k)
    orc.set_contact_data(p, s, bp, nn, k)
    assert g.last_contact_count == k
    for f in range(3):
        g.step_solve_only(1.0 / 60.0, 4, 2)
        orc.step_solve_only(1.0 / 60.0, 4, 2)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"solve-only positions {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"solve-only velocities {f}")


def test_deltas_with_diagnostics():
    sc = small_pile(8)
    cfg = config_for(sc, enable_diagnostics=True)
    g, orc = make_pair(sc, cfg)
    for _ in range(3):
        g.step(1.0 / 60.0, 10, 2)
        orc.step(1.0 / 60.0, 10, 2)
    assert_bitexact(g.get_deltas(), orc.get_deltas(), "deltas")
    assert g.get_diag_pair_count() > 0
    pairs = g.get_diag_pairs()
    assert len(pairs) == min(g.get_diag_pair_count(), cfg.max_diag_pairs)
    assert {"i", "j", "dist", "err", "normal", "lambda_f", "delta_i", "iter_index"} <= set(pairs[0])
    g.reset_diag_buffers()
    assert g.get_diag_pair_count() == 0


def test_update_mesh_bitexact():
    sc = mesh_pile(12, 24)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    v0 = sc.meshes[0][0]
    for f in range(4):
        v = v0.copy()
        v[:, 2] += 0.01 * (f + 1)
        vel = np.zeros_like(v)
        vel[:, 2] = 0.6
        g.update_mesh(0, v, vel)
        orc.update_mesh(0, v, vel)
        g.step(1.0 / 60.0, 5, 1)
        orc.step(1.0 / 60.0, 5, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"animated mesh positions {f}")


def test_determinism_run_to_run():
    sc = mesh_pile(16, 32)
    cfg = config_for(sc)
    outs = []
    for _ in range(2):
        g, _o = make_pair(sc, cfg)
        for _f in range(5):
            g.step(1.0 / 60.0, 10, 1)
        outs.append((g.get_positions(), g.get_velocities()))
    assert_bitexact(outs[0][0], outs[1][0], "run-to-run positions")
    assert_bitexact(outs[0][1], outs[1][1], "run-to-run velocities")


def test_tolerance_floor():
    """Stated tolerance of the reference port: 1e-5 relative per substep (kept as a floor)."""
    sc = small_pile(8)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.step(1.0 / 60.0, 1, 1)
    orc.step(1.0 / 60.0, 1, 1)
    a, b = g.get_positions(), orc.get_positions()
    assert np.all(np.abs(a - b) <= 1e-5 * np.maximum(np.abs(b), 1e-3))


def test_particle_exactly_on_mesh_surface_bitexact():
    import scenes

    sc = scenes.particles_on_mesh(dims=(1, 1, 1))
    sc.positions = np.array([[0.23391318321228027, -0.32021233439445496, 0.045575764030218124]], np.float32)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    g.collide_only()
    orc.collide_only()
    c = orc.get_contacts()
    assert_bitexact(g.get_contact_body_positions(), c["body_positions"], "contact point")
    assert_bitexact(g.get_contact_normals(), c["normals"], "contact normal")
    _step_compare(g, orc, 3, 1.0 / 60.0, 10, 1, "on-surface particle")
