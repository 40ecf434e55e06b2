"""Hand-written adjoint of the substep, FP64 oracle vs central finite differences.

The throw scene at 512 particles (8^3), 6 frames x 10 substeps: long enough for
plane impacts, friction, restitution and particle contacts, short enough that
the piecewise-smooth loss has no contact switch inside the FD step (over longer
horizons the Jacobian of the Jacobi-style projection grows exponentially and
FD at any step size samples contact switches, so FD stops being a reference).
"""
import numpy as np
import pytest

import oracle as O
from helpers import config_for
import scenes

FRAMES = 6


def _scene():
    return scenes.throw(dims=(8, 8, 8))


def _run(sc, cfg_over=None, v0=None, w=None):
    o = O.OracleSolver(config_for(sc, **(cfg_over or {})), sc.n, 0, precision="f64")
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities if v0 is None else v0, sc.inv_mass if w is None else w, sc.radii,
                    sc.flags)
    o.rollout(1.0 / 60.0, 10, FRAMES)
    m = o.get_state64()[0].mean(axis=0)
    target = scenes.throw_target()
    return o, float(((m - target) ** 2).sum()), m


@pytest.fixture(scope="module")
def adjoint():
    sc = _scene()
    o, L, m = _run(sc)
    target = scenes.throw_target()
    g = o.rollout_backward(np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1)))
    return sc, g


@pytest.mark.parametrize("name,eps", [("soft_contact_mu", 1e-3), ("soft_contact_restitution", 1e-3),
                                      ("particle_mu", 3e-4)])
def test_param_gradient_matches_central_fd(adjoint, name, eps):
    sc, g = adjoint
    base = getattr(config_for(sc), name)
    fd = (_run(sc, {name: base + eps})[1] - _run(sc, {name: base - eps})[1]) / (2 * eps)
    assert abs(g[name] - fd) <= 1e-3 * abs(fd), (g[name], fd)


@pytest.mark.parametrize("axis", [0, 1])
def test_velocity_gradient_matches_central_fd(adjoint, axis):
    sc, g = adjoint
    eps = 1e-3
    d = np.zeros((sc.n, 3), np.float32)
    d[:, axis] = 1.0
    adj = float((g["v0"] * d).sum())
    fd = (_run(sc, v0=sc.velocities + eps * d)[1] - _run(sc, v0=sc.velocities - eps * d)[1]) / (2 * eps)
    assert abs(adj - fd) <= 1e-3 * abs(fd), (adj, fd)


def test_inverse_mass_gradient_matches_central_fd(adjoint):
    sc, g = adjoint
    eps = 1e-3
    d = (np.random.default_rng(0).normal(size=sc.n) * 100.0).astype(np.float32)
    adj = float((g["inv_mass"] * d).sum())
    fd = (_run(sc, w=sc.inv_mass + eps * d)[1] - _run(sc, w=sc.inv_mass - eps * d)[1]) / (2 * eps)
    assert abs(adj - fd) <= 1e-3 * abs(fd), (adj, fd)


def test_random_velocity_direction_small_step(adjoint):
    """Per-particle directions switch contacts at eps = 1e-3; at 1e-5 the FD is smooth."""
    sc, g = adjoint
    eps = 1e-5
    d = np.random.default_rng(1).normal(size=(sc.n, 3))
    adj = float((g["v0"] * d).sum())
    vp = (sc.velocities.astype(np.float64) + eps * d).astype(np.float32)
    vm = (sc.velocities.astype(np.float64) - eps * d).astype(np.float32)
    fd = (_run(sc, v0=vp)[1] - _run(sc, v0=vm)[1]) / (2 * eps)
    assert abs(adj - fd) <= 2e-2 * abs(fd), (adj, fd)  # float32 inputs quantise the 1e-5 step


def test_f32_adjoint_close_to_f64():
    sc = _scene()
    target = scenes.throw_target()
    out = {}
    for prec in ("f32", "f64"):
        o = O.OracleSolver(config_for(sc), sc.n, 0, precision=prec)
        o.finalize_meshes()
        o.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
        o.rollout(1.0 / 60.0, 10, FRAMES)
        m = o.get_positions().astype(np.float64).mean(axis=0)
        out[prec] = o.rollout_backward(np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1)))
    for k in ("soft_contact_mu", "soft_contact_restitution"):
        assert abs(out["f32"][k] - out["f64"][k]) <= 1e-2 * abs(out["f64"][k])
    a, b = out["f32"]["v0"].sum(axis=0), out["f64"]["v0"].sum(axis=0)
    assert np.allclose(a, b, rtol=1e-2, atol=1e-6)


def test_rollout_rejects_meshes():
    sc = scenes.particles_on_mesh(dims=(2, 2, 2), hf_vertices=8)
    o = O.OracleSolver(config_for(sc), sc.n, 0)
    v, t, m, wt = sc.meshes[0]
    o.add_mesh(v, t, m, None, wt)
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    with pytest.raises(RuntimeError):
        o.rollout(1.0 / 60.0, 10, 1)


def _run_frames(sc, frames, prec="f64", cfg_over=None, v0=None):
    o = O.OracleSolver(config_for(sc, **(cfg_over or {})), sc.n, 0, precision=prec)
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities if v0 is None else v0, sc.inv_mass, sc.radii, sc.flags)
    o.rollout(1.0 / 60.0, 10, frames)
    x = o.get_state64()[0] if prec == "f64" else o.get_positions().astype(np.float64)
    m = x.mean(axis=0)
    target = scenes.throw_target()
    return o, float(((m - target) ** 2).sum()), m


def test_fd_matches_at_70_substeps():
    """The longest horizon of the 512-particle copy at which central differences at eps 1e-3
    still match the exact gradient to 1e-3 (the block has just landed; measured 2e-4 for the
    plane friction, 1e-5 for a uniform velocity shift). At 80 substeps eps 1e-3 straddles a
    contact switch and only eps 1e-4 matches; from 90 on no step size does."""
    sc = _scene()
    o, _, m = _run_frames(sc, 7)
    target = scenes.throw_target()
    g = o.rollout_backward(np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1)))
    eps = 1e-3
    fd_mu = (_run_frames(sc, 7, cfg_over={"soft_contact_mu": 0.5 + eps})[1] -
             _run_frames(sc, 7, cfg_over={"soft_contact_mu": 0.5 - eps})[1]) / (2 * eps)
    assert abs(g["soft_contact_mu"] - fd_mu) <= 1e-3 * abs(fd_mu), (g["soft_contact_mu"], fd_mu)
    d = np.zeros((sc.n, 3), np.float32)
    d[:, 0] = 1.0
    fd_v = (_run_frames(sc, 7, v0=sc.velocities + eps * d)[1] - _run_frames(sc, 7, v0=sc.velocities - eps * d)[1]) / (
        2 * eps)
    assert abs(float((g["v0"] * d).sum()) - fd_v) <= 1e-3 * abs(fd_v)


def test_gradient_growth_beyond_the_fd_horizon_is_genuine():
    """Past ~80 substeps the exact gradient of the throw grows exponentially (the Jacobian of the
    Jacobi-style contact projection in the settled pile has modes above 1 per substep). Not an
    FP32 artefact: the FP64 and FP32 adjoints reach the same magnitude at 240 substeps, and the
    central difference, bounded over a finite step, grows toward it as the step shrinks."""
    sc = _scene()
    target = scenes.throw_target()
    norms = {}
    for prec in ("f64", "f32"):
        o, _, m = _run_frames(sc, 24, prec)
        g = o.rollout_backward(np.tile((2.0 * (m - target) / sc.n).astype(np.float32), (sc.n, 1)))
        norms[prec] = float(np.linalg.norm(g["v0"]))
    assert norms["f64"] > 1e5, norms
    assert norms["f64"] / 3 < norms["f32"] < norms["f64"] * 3, norms
    d = np.zeros((sc.n, 3), np.float32)
    d[:, 0] = 1.0
    fd = {}
    for eps in (1e-3, 1e-6):
        fd[eps] = (_run_frames(sc, 24, v0=sc.velocities + eps * d)[1] -
                   _run_frames(sc, 24, v0=sc.velocities - eps * d)[1]) / (2 * eps)
    assert abs(fd[1e-6]) > 10 * abs(fd[1e-3]), fd
