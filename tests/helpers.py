"""Builds the same seeded scene on the CUDA path (vkxpbd) and on the CPU oracle."""
from __future__ import annotations

import numpy as np

import oracle as O
import scenes


def config_for(scene, gpu=True, **overrides):
    """The scene's configuration on vkxpbd.SolverConfig, or (gpu=False) on the oracle's own
    SolverConfig with the same defaults (no product code loaded)."""
    if gpu:
        import vkxpbd

        cfg = vkxpbd.SolverConfig()
    else:
        cfg = O.SolverConfig()
    scene.apply_config(cfg)
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def make_pair(scene, cfg, max_contacts=0, gpu=True, precision="f32", body_params=None):
    """(gpu solver or None, oracle solver) with identical inputs. gpu=False loads no product code."""
    if gpu:
        import vkxpbd

    body_params = dict(body_params or {})
    orc = O.OracleSolver(cfg, scene.n, max_contacts, precision=precision)
    g = None
    if gpu:
        g = vkxpbd.XpbdSolver()
        g.init(cfg, scene.n, max_contacts)
    for (v, t, margin, wt) in scene.meshes:
        orc.add_mesh(v, t, margin, None, wt)
        if g is not None:
            g.add_mesh(v, t, shape_margin=margin, is_watertight=wt)
    orc.finalize_meshes()
    if g is not None:
        g.finalize_meshes()
    if getattr(scene, "bodies", None) is not None:
        b = scene.bodies
        bargs = (b.q, b.qd, b.com, b.inertia, b.inv_inertia, b.inv_mass, b.flags)
        orc.set_bodies(*bargs)
        orc.set_body_params(**body_params)
        if g is not None:
            g.set_bodies(*bargs)
            g.set_body_params(**body_params)
    args = (scene.positions, scene.velocities, scene.inv_mass, scene.radii, scene.flags)
    orc.set_particles(*args)
    if g is not None:
        g.set_particles(*args)
    return g, orc


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_bitexact(a, b, what=""):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if not np.array_equal(bits(a), bits(b)):
        diff = np.nonzero(bits(a).reshape(-1) != bits(b).reshape(-1))[0]
        af, bf = a.reshape(-1), b.reshape(-1)
        k = diff[0]
        raise AssertionError(f"{what}: {diff.size} of {af.size} words differ; first at {k}: {af[k]!r} vs {bf[k]!r}; "
                             f"max abs diff {np.max(np.abs(af.astype(np.float64) - bf.astype(np.float64)))}")


def small_pile(n_side=8, **kw):
    return scenes.pile(dims=(n_side, n_side, n_side), **kw)


def mesh_pile(n_side=16, hf=32, **kw):
    sc = scenes.pile(dims=(n_side, n_side, n_side), spacing=0.01, radius=0.005, jitter=0.001, bottom_z=0.12, **kw)
    v, t = scenes.heightfield(hf, extent=0.4, amplitude=0.02)
    sc.meshes.append((v, t, 0.0, None))
    return sc


def box_scene(n_side=6, boxes=((0.05, 0.04, 0.03),), positions=((0.0, 0.0, 0.25),), seed=3, hf=None, **kw):
    """A small particle pile plus dynamic boxes (random orientations) dropped from above."""
    sc = scenes.pile(dims=(n_side, n_side, n_side), spacing=0.01, radius=0.005, jitter=0.001, bottom_z=0.02, **kw)
    if hf:
        v, t = scenes.heightfield(hf, extent=0.4, amplitude=0.02)
        sc.meshes.append((v, t, 0.0, None))
    rng = np.random.default_rng(seed)
    return scenes.add_boxes(sc, list(boxes), list(positions), scenes.random_quats(len(boxes), rng))
