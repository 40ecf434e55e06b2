"""GPU adjoint (xpbd_rollout_backward, vkxpbd.diff) vs the CPU oracle's adjoint."""
import numpy as np
import pytest

import oracle as O
from helpers import assert_bitexact, config_for
import scenes

pytestmark = pytest.mark.gpu

FRAMES = 6


def _loss_grad(x, target):
    m = x.astype(np.float64).mean(axis=0)
    return float(((m - target) ** 2).sum()), np.tile((2.0 * (m - target) / x.shape[0]).astype(np.float32),
                                                      (x.shape[0], 1))


def _gpu(sc, cfg, frames=FRAMES, ckpt=2):
    import vkxpbd

    g = vkxpbd.XpbdSolver()
    g.init(cfg, sc.n)
    g.finalize_meshes()
    g.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    g.rollout(1.0 / 60.0, 10, frames, 1, ckpt)
    return g


def _oracle(sc, cfg, prec, frames=FRAMES):
    o = O.OracleSolver(cfg, sc.n, 0, precision=prec)
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities, sc.inv_mass, sc.radii, sc.flags)
    o.rollout(1.0 / 60.0, 10, frames)
    return o


def test_rollout_forward_bitexact_and_adjoint_matches_oracle():
    sc = scenes.throw(dims=(8, 8, 8))
    cfg = config_for(sc)
    target = scenes.throw_target()
    g = _gpu(sc, cfg)
    o = _oracle(sc, cfg, "f32")
    assert_bitexact(g.get_positions(), o.get_positions(), "rollout final positions")
    _, gx = _loss_grad(g.get_positions(), target)
    gg = g.rollout_backward(gx)
    go = o.rollout_backward(gx)
    for k in ("soft_contact_mu", "particle_mu", "soft_contact_restitution"):
        assert abs(gg[k] - go[k]) <= 1e-3 * abs(go[k]) + 1e-12, (k, gg[k], go[k])
    for k in ("v0", "x0", "inv_mass"):
        a, b = gg[k].astype(np.float64), go[k]
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b), k
    # the solver is left at the rollout's final state
    assert_bitexact(g.get_positions(), o.get_positions(), "state after backward")


def test_adjoint_close_to_f64_oracle():
    sc = scenes.throw(dims=(8, 8, 8))
    cfg = config_for(sc)
    target = scenes.throw_target()
    g = _gpu(sc, cfg)
    o = _oracle(sc, cfg, "f64")
    _, gx = _loss_grad(g.get_positions(), target)
    gg, go = g.rollout_backward(gx), o.rollout_backward(gx)
    for k in ("soft_contact_mu", "soft_contact_restitution"):
        assert abs(gg[k] - go[k]) <= 1e-2 * abs(go[k]), (k, gg[k], go[k])
    assert np.allclose(gg["v0"].sum(axis=0), go["v0"].sum(axis=0), rtol=1e-2, atol=1e-6)


def test_checkpoint_spacing_does_not_change_gradients():
    sc = scenes.throw(dims=(6, 6, 6))
    cfg = config_for(sc)
    target = scenes.throw_target()
    res = []
    for ckpt in (1, 2, 4):
        g = _gpu(sc, cfg, frames=4, ckpt=ckpt)
        _, gx = _loss_grad(g.get_positions(), target)
        res.append(g.rollout_backward(gx))
    for r in res[1:]:
        assert_bitexact(r["v0"], res[0]["v0"], "v0 gradient")
        assert_bitexact(r["inv_mass"], res[0]["inv_mass"], "inverse-mass gradient")
        assert r["soft_contact_mu"] == res[0]["soft_contact_mu"]


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from vkxpbd.diff import DiffSim

    sc = scenes.throw(dims=(6, 6, 6))
    cfg = config_for(sc)
    target = torch.tensor(scenes.throw_target())
    sim = DiffSim(cfg, sc.radii, dt=1.0 / 60.0, substeps=10, frames=4, checkpoint_frames=2)
    v0 = torch.tensor(sc.velocities, requires_grad=True)
    w = torch.tensor(sc.inv_mass, requires_grad=True)
    mu = torch.tensor(float(cfg.soft_contact_mu), requires_grad=True)
    e = torch.tensor(float(cfg.soft_contact_restitution), requires_grad=True)
    kmu = torch.tensor(float(cfg.particle_mu), requires_grad=True)
    x = sim(torch.tensor(sc.positions), v0, w, mu, kmu, e)
    loss = ((x.double().mean(0) - target) ** 2).sum()
    loss.backward()
    # same numbers as the direct binding
    g = _gpu(sc, cfg, frames=4)
    _, gx = _loss_grad(g.get_positions(), scenes.throw_target())
    gg = g.rollout_backward(gx)
    assert np.allclose(v0.grad.numpy(), gg["v0"], rtol=1e-5, atol=1e-9)
    assert abs(float(mu.grad) - gg["soft_contact_mu"]) <= 1e-5 * abs(gg["soft_contact_mu"]) + 1e-12
    assert np.allclose(w.grad.numpy(), gg["inv_mass"], rtol=1e-5, atol=1e-12)
    # central differences (eps 1e-3) of the FP64 oracle's forward for the friction coefficient
    # and a uniform velocity shift: the float32 forward cannot resolve a 2e-3 step of the loss
    eps = 1e-3
    fd_mu = (_loss64(sc, 4, soft_contact_mu=0.5 + eps) - _loss64(sc, 4, soft_contact_mu=0.5 - eps)) / (2 * eps)
    assert abs(float(mu.grad) - fd_mu) <= 1e-3 * abs(fd_mu), (float(mu.grad), fd_mu)
    d = np.zeros((sc.n, 3), np.float32)
    d[:, 0] = 1.0
    fd_v = (_loss64(sc, 4, v0=sc.velocities + eps * d) - _loss64(sc, 4, v0=sc.velocities - eps * d)) / (2 * eps)
    adj_v = float((v0.grad.numpy().astype(np.float64) * d).sum())
    assert abs(adj_v - fd_v) <= 1e-3 * abs(fd_v), (adj_v, fd_v)


def _loss64(sc, frames, v0=None, **over):
    """Loss of the FP64 oracle's rollout (the finite-difference reference)."""
    o = O.OracleSolver(config_for(sc, **over), sc.n, 0, precision="f64")
    o.finalize_meshes()
    o.set_particles(sc.positions, sc.velocities if v0 is None else v0, sc.inv_mass, sc.radii, sc.flags)
    o.rollout(1.0 / 60.0, 10, frames)
    m = o.get_state64()[0].mean(axis=0)
    return float(((m - scenes.throw_target()) ** 2).sum())


def test_full_throw_gradient_matches_fd_at_60_substeps():
    """The 32,768-particle throw: the GPU adjoint (FP32, split hash-grid keys) against central
    differences (eps 1e-3) of the FP64 oracle's forward at 60 substeps — the longest horizon at
    which differences at this step still match the exact gradient (at 70 the plane friction's
    already differs by 2e-3; past ~80 substeps the gradient grows exponentially, see
    test_cpu_adjoint). Plane friction and uniform velocity shifts to 1e-3 relative; restitution
    to 3e-3 (its term is small, -4e-7, and the FP32 adjoint's rounding leaves 2e-3 where the
    FP64 adjoint matches to 2e-6). The particle-friction gradient is left out: the friction
    branches of the dense contact set switch inside any step of 3e-5 or more, so differences
    do not converge, and FP32 and FP64 forwards take different branches (adjoints 16% apart)."""
    sc = scenes.throw()
    cfg = config_for(sc)
    g = _gpu(sc, cfg, frames=6)
    _, gx = _loss_grad(g.get_positions(), scenes.throw_target())
    gg = g.rollout_backward(gx)
    eps = 1e-3
    for name, tol in (("soft_contact_mu", 1e-3), ("soft_contact_restitution", 3e-3)):
        base = getattr(cfg, name)
        fd = (_loss64(sc, 6, **{name: base + eps}) - _loss64(sc, 6, **{name: base - eps})) / (2 * eps)
        assert abs(gg[name] - fd) <= tol * abs(fd), (name, gg[name], fd)
    for axis in (0, 1):
        d = np.zeros((sc.n, 3), np.float32)
        d[:, axis] = 1.0
        fd = (_loss64(sc, 6, v0=sc.velocities + eps * d) - _loss64(sc, 6, v0=sc.velocities - eps * d)) / (2 * eps)
        adj = float((gg["v0"].astype(np.float64) * d).sum())
        assert abs(adj - fd) <= 1e-3 * abs(fd), (axis, adj, fd)
