"""The three forms of the solve kernel against each other and the oracle.

The solve kernel computes each particle's particle-particle total per thread (each thread the
pair terms of its own neighbours), per warp (the lanes filter their own candidates, then
compute all buffered pair terms of the warp together and each lane adds its own in candidate
order), or per thread from a block's neighbourhood records staged in shared memory. All sum
the same terms in the same order, so solvers forced to any form, and one choosing by timing,
must agree bit for bit with the oracle: inactive, proxy and kinematic particles with cohesion
and adhesion over two iterations, a heightfield with the split first iteration, dynamic
boxes, batched scenes (which the staged form leaves to the global path), and a pile large
enough for split grid keys.
"""
import numpy as np
import pytest

import scenes
from helpers import assert_bitexact, box_scene, config_for, make_pair, mesh_pile, small_pile

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
FORMS = (0, 1, 2, 3)


def _run(sc, cfg, frames, substeps, iterations, what, split=None, body_params=None):
    gpus = []
    orc = None
    for form in FORMS:
        g, o = make_pair(sc, cfg, body_params=body_params)
        g.set_solve_form(form)
        if split is not None:
            g.set_solve_split(split)
        assert g.solve_form == form
        gpus.append(g)
        orc = orc or o
    for f in range(frames):
        orc.step(DT, substeps, iterations)
        for form, g in enumerate(gpus):
            g.step(DT, substeps, iterations)
            assert_bitexact(g.get_positions(), orc.get_positions(), f"{what} form {form} positions frame {f}")
            assert_bitexact(g.get_velocities(), orc.get_velocities(), f"{what} form {form} velocities frame {f}")
            assert g.last_contact_count == orc.last_contact_count, f"{what} form {form} contacts frame {f}"
    return gpus, orc


def test_forms_flags_cohesion_two_iterations():
    sc = small_pile(11)
    n = sc.n
    flags = np.ones(n, np.int32)
    flags[::7] = 0          # inactive
    flags[3::11] = 3        # active + proxy
    sc.flags = flags
    sc.inv_mass[::13] = 0.0  # kinematic
    cfg = config_for(sc, particle_cohesion=0.002, particle_adhesion=0.001, soft_contact_restitution=0.5)
    _run(sc, cfg, 6, 5, 2, "flags")


@pytest.mark.parametrize("split", [0, 1])
def test_forms_heightfield(split):
    sc = mesh_pile(16, 32)
    cfg = config_for(sc)
    _run(sc, cfg, 12, 10, 1, f"heightfield split={split}", split=split)


def test_forms_boxes():
    sc = box_scene(n_side=8, positions=((0.035, 0.035, 0.12),))
    cfg = config_for(sc)
    gpus, orc = _run(sc, cfg, 15, 10, 1, "boxes")
    for g in gpus:
        assert_bitexact(g.get_body_q(), orc.get_body_q(), "boxes body q")


def test_forms_batched_scenes():
    counts = [700, 1, 2048, 64, 1500, 333]
    batch = scenes.Batch([scenes.pile_of(c, seed=46 + s) for s, c in enumerate(counts)])
    cfg = config_for(batch)
    import vkxpbd

    oracles = [make_pair(sc, cfg, gpu=False)[1] for sc in batch.scenes]
    gs = []
    for form in FORMS:
        g = vkxpbd.XpbdSolver()
        g.init_batched(cfg, batch.counts)
        g.finalize_meshes()
        g.set_particles(batch.concat("positions"), batch.concat("velocities"), batch.concat("inv_mass"),
                        batch.concat("radii"), batch.concat("flags"))
        g.set_solve_form(form)
        gs.append(g)
    off = gs[0].scene_offsets()
    for f in range(5):
        for g in gs:
            g.step(DT, 10, 1)
        for s, orc in enumerate(oracles):
            orc.step(DT, 10, 1)
            for form, g in enumerate(gs):
                assert_bitexact(g.get_positions()[off[s]:off[s + 1]], orc.get_positions(),
                                f"batched form {form} scene {s} frame {f}")


def test_timed_form_choice_is_exact():
    """A solver of 16,384 particles or more times both forms after its first frame and keeps
    the faster; the state stays bit-exact through the timing launches."""
    sc = scenes.pile_of(20_000)
    cfg = config_for(sc)
    g, orc = make_pair(sc, cfg)
    for f in range(4):
        g.step(DT, 10, 1)
        orc.step(DT, 10, 1)
        assert_bitexact(g.get_positions(), orc.get_positions(), f"timed form frame {f}")
        assert_bitexact(g.get_velocities(), orc.get_velocities(), f"timed form frame {f}")
    assert g.solve_form in FORMS
    with pytest.raises(RuntimeError, match="set_solve_form"):
        g.set_solve_form(4)


def test_forms_split_keys_pile():
    """40,000 particles (split grid keys): most blocks stage their rows in the staged form."""
    sc = scenes.pile_of(40_000)
    cfg = config_for(sc)
    _run(sc, cfg, 4, 10, 1, "split-key pile")
