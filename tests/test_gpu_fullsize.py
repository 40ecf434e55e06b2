"""The timed workloads at their full sizes, bit for bit against the CPU oracle.

The other GPU tests pin every path on small scenes; these run the exact scenes the benchmark
times (the reference's step loop, src/scene.cpp:698-1092), so that every measured number is
a number for checked code:

- particles on a mesh: 262,144 particles on the 130,050-triangle heightfield; one-scene
  solvers of this size sort split hash-grid keys by default (no override);
- mixed: 1,048,576 particles and 1,024 dynamic boxes on the plane and the heightfield, the
  first frame and a frame after the benchmark's 20-frame pre-roll;
- batched: all 512 uneven scenes with 0-16 boxes each in one batched solver, the first frame
  and a frame after a pre-roll in which the boxes land, compared scene by scene with the
  oracle stepping each scene alone;
- differentiable throw: 32,768 particles over the full 600 substeps, and the adjoint of the
  first 60 substeps against the oracle's adjoint.

Where the oracle would take minutes the comparison is cut by substeps or frames, never by
particles. A pre-rolled state is the GPU's, uploaded to the oracle (the step's result depends
only on the particle and body state, the meshes and the configuration).
"""
import numpy as np
import pytest

import oracle as O
import scenes
from helpers import assert_bitexact, config_for, make_pair

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


@pytest.fixture(autouse=True, scope="module")
def _all_threads():
    import os

    O.load("f32").or_set_threads(os.cpu_count() or 1)
    O.load("f64").or_set_threads(os.cpu_count() or 1)


def _compare_frame(g, orc, what, bodies=False):
    g.step(DT, 10, 1)
    orc.step(DT, 10, 1)
    assert_bitexact(g.get_positions(), orc.get_positions(), f"{what} positions")
    assert_bitexact(g.get_velocities(), orc.get_velocities(), f"{what} velocities")
    assert g.last_contact_count == orc.last_contact_count, f"{what} contact count"
    if bodies:
        assert_bitexact(g.get_body_q(), orc.get_body_q(), f"{what} body q")
        assert_bitexact(g.get_body_qd(), orc.get_body_qd(), f"{what} body qd")


def test_particles_on_mesh_full_size():
    sc = scenes.particles_on_mesh()
    assert sc.n == 262_144 and sc.meshes[0][1].shape[0] == 130_050
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    _compare_frame(g, orc, "first frame")
    for _ in range(29):  # the benchmark's pre-roll: the pile lies on the heightfield
        g.step(DT, 10, 1)
    orc.set_particles(g.get_positions(), g.get_velocities())
    for f in range(5):
        _compare_frame(g, orc, f"frame {31 + f}")
    assert g.last_contact_count > 50_000  # the pile lies on the heightfield (76,104 measured)


def test_mixed_full_size():
    sc = scenes.mixed()
    assert sc.n == 1_048_576 and len(sc.meshes) == 1 + 1024
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    _compare_frame(g, orc, "first frame", bodies=True)
    for _ in range(19):  # the benchmark's 20-frame pre-roll: boxes land in the pile
        g.step(DT, 10, 1)
    orc.set_particles(g.get_positions(), g.get_velocities())
    orc.set_bodies(g.get_body_q(), g.get_body_qd())
    _compare_frame(g, orc, "frame 21", bodies=True)
    assert g.last_contact_count > 150_000  # boxes and heightfield in contact (236,105 measured)
    assert np.isfinite(g.get_body_q()).all()


def _batched_solver(batch, cfg):
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
    return g, body_scene


def _compare_batched_frame(g, batch, cfg, body_scene, x0, v0, q0, qd0, what):
    """One frame of the batched solver against each scene stepped alone by the oracle from the
    same state (scene s: its particles, the shared anchor body and its own boxes)."""
    g.step(DT, 10, 1)
    x, v, q, qd = g.get_positions(), g.get_velocities(), g.get_body_q(), g.get_body_qd()
    off = g.scene_offsets()
    for s, sc in enumerate(batch.scenes):
        _, orc = make_pair(sc, cfg, gpu=False)
        a, b = off[s], off[s + 1]
        orc.set_particles(x0[a:b], v0[a:b])
        rows = np.concatenate([[0], np.nonzero(body_scene == s)[0]])
        orc.set_bodies(q0[rows], qd0[rows])
        orc.step(DT, 10, 1)
        assert_bitexact(x[a:b], orc.get_positions(), f"{what} scene {s} positions")
        assert_bitexact(v[a:b], orc.get_velocities(), f"{what} scene {s} velocities")
        assert_bitexact(q[rows], orc.get_body_q(), f"{what} scene {s} body q")
        assert_bitexact(qd[rows], orc.get_body_qd(), f"{what} scene {s} body qd")
        del orc


def test_batched_512_scenes_full_size():
    batch = scenes.batched_piles_with_boxes(512, max_boxes=16)
    cfg = config_for(batch)
    g, body_scene = _batched_solver(batch, cfg)
    assert g.scene_count() == 512 and (body_scene >= 0).sum() > 3000
    state = (g.get_positions(), g.get_velocities(), g.get_body_q(), g.get_body_qd())
    _compare_batched_frame(g, batch, cfg, body_scene, *state, "first frame")
    for _ in range(39):  # the boxes fall 0.2-3.4 m onto their piles
        g.step(DT, 10, 1)
    state = (g.get_positions(), g.get_velocities(), g.get_body_q(), g.get_body_qd())
    _compare_batched_frame(g, batch, cfg, body_scene, *state, "frame 41")


def test_throw_600_substeps_and_adjoint_full_size():
    import vkxpbd

    sc = scenes.throw()
    assert sc.n == 32_768
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    for f in range(60):  # 600 substeps, bit-exact at every frame
        g.step(DT, 10, 1)
        orc.step(DT, 10, 1)
        if f % 10 == 9 or f == 0:
            assert_bitexact(g.get_positions(), orc.get_positions(), f"throw positions frame {f}")
            assert_bitexact(g.get_velocities(), orc.get_velocities(), f"throw velocities frame {f}")
    # adjoint of the first 60 substeps (checkpointed every 20) against the oracle's FP32 adjoint
    target = scenes.throw_target()
    s = vkxpbd.XpbdSolver()
    s.init(cfg, sc.n)
    s.finalize_meshes()
    s.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    s.rollout(DT, 10, 6, 1, 2)
    o = O.OracleSolver(cfg, sc.n, 0, precision="f32")
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    o.rollout(DT, 10, 6)
    x = s.get_positions()
    assert_bitexact(x, o.get_positions(), "rollout final positions")
    m = x.astype(np.float64).mean(axis=0)
    gx = np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1))
    gg, go = s.rollout_backward(gx), o.rollout_backward(gx)
    for k in ("soft_contact_mu", "particle_mu", "soft_contact_restitution"):
        assert abs(gg[k] - go[k]) <= 1e-3 * abs(go[k]) + 1e-12, (k, gg[k], go[k])
    for k in ("v0", "x0", "inv_mass"):
        a, b = gg[k].astype(np.float64), go[k]
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b), k
