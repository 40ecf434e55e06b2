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
    # central FD of the GPU forward for the friction coefficient
    eps = 1e-3
    with torch.no_grad():
        lp = ((sim(torch.tensor(sc.positions), v0, w, mu + eps, kmu, e).double().mean(0) - target) ** 2).sum()
        lm = ((sim(torch.tensor(sc.positions), v0, w, mu - eps, kmu, e).double().mean(0) - target) ** 2).sum()
    fd = float(lp - lm) / (2 * eps)
    assert abs(float(mu.grad) - fd) <= 2e-2 * abs(fd), (float(mu.grad), fd)
