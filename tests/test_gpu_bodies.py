"""Dynamic rigid bodies (boxes as body-frame meshes) vs the CPU oracle.

Covers integrate_bodies.comp, apply_body_deltas.comp and
solve_body_contact_positions.comp, the body deltas of particle contacts
(solve_particle_shape_contacts.comp:193-199) and the rigid contact generator.
Bar: bit-exact particle and body states every frame.
"""
import numpy as np
import pytest

from helpers import assert_bitexact, box_scene, config_for, make_pair

pytestmark = pytest.mark.gpu


def _run(sc, frames, substeps=10, iterations=1, body_params=None, **cfg_kw):
    cfg = config_for(sc, **cfg_kw)
    g, orc = make_pair(sc, cfg, body_params=body_params)
    for f in range(frames):
        g.step(1.0 / 60.0, substeps, iterations)
        orc.step(1.0 / 60.0, substeps, iterations)
        assert_bitexact(g.get_body_q(), orc.get_body_q(), f"body q frame {f}")
        assert_bitexact(g.get_body_qd(), orc.get_body_qd(), f"body qd frame {f}")
        assert_bitexact(g.get_positions(), orc.get_positions(), f"positions frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"velocities frame {f}")
    return g, orc


def test_box_on_plane_bitexact():
    sc = box_scene(n_side=2, positions=((0.3, 0.0, 0.2),))
    g, _ = _run(sc, 40)
    # the box comes to rest on its smallest face (half extent 0.03)
    q = g.get_body_q()[-1]
    assert abs(q[2] - 0.03) < 2e-3


def test_box_on_particles_bitexact():
    """A box lands on a particle pile: particle contacts on a moving mesh, body deltas."""
    sc = box_scene(n_side=8, positions=((0.035, 0.035, 0.2),))
    _run(sc, 30)


def test_boxes_stack_and_heightfield_bitexact():
    """Box-box rigid contacts (both roles), boxes on a static heightfield, 2 iterations."""
    sc = box_scene(n_side=4, boxes=((0.05, 0.05, 0.03), (0.04, 0.03, 0.03), (0.03, 0.03, 0.03)),
                   positions=((0.0, 0.0, 0.12), (0.01, 0.0, 0.25), (0.2, 0.1, 0.15)), hf=24)
    _run(sc, 25, substeps=5, iterations=2, body_params=dict(rigid_mu_torsional=0.01, rigid_mu_rolling=0.01))


def test_mixed_small_bitexact():
    """A scaled-down particles + heightfield + falling boxes scene (the mixed workload's recipe)."""
    import scenes

    sc = scenes.mixed(dims=(24, 24, 12), n_boxes=24, hf_vertices=64)
    _run(sc, 20)


def test_particle_weighting_off_bitexact():
    sc = box_scene(n_side=8, positions=((0.035, 0.035, 0.12),))
    _run(sc, 10, body_params=dict(particle_contact_con_weighting=0, rigid_contact_con_weighting=0))


def test_box_shell_grid_collisions_bitexact():
    """Particles in a shell around one large box (radii up to 0.012 above particle_max_radius).
    With one dynamic body the box grid has 64 buckets for up to 64 cells, so the box's own
    cells collide in the hash; each particle must still take the box exactly once, and the
    grid's reach must cover the largest radius set."""
    sc = box_scene(n_side=2, boxes=((0.08, 0.06, 0.05),), positions=((0.0, 0.0, 0.3),))
    rng = np.random.default_rng(9)
    n = 2500
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = np.array([0.0, 0.0, 0.3]) + d * rng.uniform(0.05, 0.13, (n, 1))
    sc.positions = pos.astype(np.float32)
    sc.velocities = np.zeros_like(sc.positions)
    sc.inv_mass = np.full(n, 1000.0, np.float32)
    sc.radii = rng.uniform(0.003, 0.012, n).astype(np.float32)
    sc.flags = np.ones(n, np.int32)
    _run(sc, 3, substeps=4)


def test_particles_between_eight_boxes_bitexact():
    """Particles in the gap between eight small boxes: each particle has up to eight
    candidate moving meshes, past the per-particle share the query kernel lists for the
    warp (the rest are queried by the particle's own lane, in candidate order)."""
    he, c = 0.02, 0.0215
    pos = [(sx * c, sy * c, 0.3 + sz * c) for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]
    sc = box_scene(n_side=2, boxes=[(he, he, he)] * 8, positions=pos, seed=5)
    rng = np.random.default_rng(21)
    n = 600
    p = (rng.random((n, 3)) - 0.5) * 0.012 + np.array([0.0, 0.0, 0.3])
    sc.positions = p.astype(np.float32)
    sc.velocities = np.zeros_like(sc.positions)
    sc.inv_mass = np.full(n, 1000.0, np.float32)
    sc.radii = np.full(n, 0.004, np.float32)
    sc.flags = np.ones(n, np.int32)
    _run(sc, 3, substeps=4)


def _icosphere(radius, subdivisions=1):
    """Closed triangle mesh of a sphere: an icosahedron with each face split in four (80)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    for _ in range(subdivisions):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                c = verts[a] + verts[b]
                verts.append(c / np.linalg.norm(c))
                mid[k] = len(verts) - 1
            return mid[k]

        f = [g for (a, b, c) in f for g in ((a, m(a, b), m(c, a)), (b, m(b, c), m(a, b)), (c, m(c, a), m(b, c)),
                                            (m(a, b), m(b, c), m(c, a)))]
    return (np.array(verts) * radius).astype(np.float32), np.array(f, np.uint32)


def test_dynamic_mesh_larger_than_a_box_bitexact():
    """A dynamic body whose mesh has 80 triangles (an icosphere) dropped on a particle pile: its
    particle queries take the per-thread traversal with the shader's 32-entry stack, the boxes
    of the other tests the shared-memory stack of small meshes."""
    import scenes

    sc = box_scene(n_side=8, positions=((0.035, 0.035, 0.2),))
    v, t = _icosphere(0.04)
    b = sc.bodies
    sc.meshes.append((v, t, 0.0, True))
    nb = len(sc.meshes)
    nbod = scenes.Bodies.static(nb)
    for name in ("q", "qd", "com", "inertia", "inv_inertia", "inv_mass", "flags"):
        getattr(nbod, name)[: nb - 1] = getattr(b, name)
    m = 1000.0 * 4.0 / 3.0 * np.pi * 0.04 ** 3
    inertia = np.eye(3) * 0.4 * m * 0.04 ** 2
    nbod.q[nb - 1] = (-0.03, -0.02, 0.16, 0.0, 0.0, 0.0, 1.0)
    nbod.inertia[nb - 1] = inertia
    nbod.inv_inertia[nb - 1] = np.linalg.inv(inertia)
    nbod.inv_mass[nb - 1] = 1.0 / m
    sc.bodies = nbod
    _run(sc, 25)


def test_set_bodies_state_in_place_and_dynamic_set_change_bitexact():
    """set_bodies with the same dynamic bodies (a new state of the same scene, as a driver
    restoring a frame does every step) uploads the state in place and keeps the tables and
    graphs; a change of which bodies are dynamic rebuilds them. Both stay bit-exact."""
    sc = box_scene(n_side=6, boxes=((0.05, 0.04, 0.03), (0.04, 0.03, 0.03)),
                   positions=((0.0, 0.0, 0.15), (0.12, 0.02, 0.2)))
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    dt = 1.0 / 60.0

    def both(frames, what):
        for f in range(frames):
            g.step(dt, 10, 1)
            orc.step(dt, 10, 1)
            assert_bitexact(g.get_body_q(), orc.get_body_q(), f"{what} body q frame {f}")
            assert_bitexact(g.get_positions(), orc.get_positions(), f"{what} positions frame {f}")

    both(4, "start")
    q, qd = orc.get_body_q(), orc.get_body_qd()
    x, v = orc.get_positions(), orc.get_velocities()
    for _ in range(3):  # restore the same state, step, restore: the in-place path every time
        g.set_particles(x, v)
        g.set_bodies(q, qd)
        g.step(dt, 10, 1)
    g.set_particles(x, v)
    g.set_bodies(q, qd)
    orc.set_particles(x, v)
    orc.set_bodies(q, qd)
    both(3, "restored")
    inv_mass = np.array(sc.bodies.inv_mass, np.float32).copy()
    inv_mass[-1] = 0.0  # the second box becomes static: the tables are rebuilt
    g.set_bodies(inv_mass=inv_mass)
    orc.set_bodies(inv_mass=inv_mass)
    both(3, "one box static")
