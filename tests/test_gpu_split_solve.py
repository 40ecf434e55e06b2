"""The first solver iteration split around contact generation vs fused after it.

With meshes, the first iteration's particle-particle part can run beside contact
generation (its totals kept per particle) and the rest of the iteration after it. Both
forms add the same totals to the shape deltas in the same order, so a solver forced to
either form, and one choosing by timing, must agree bit for bit with each other and with
the oracle: static heightfield, and dynamic boxes with a heightfield (bodies).
"""
import pytest

from helpers import assert_bitexact, box_scene, config_for, make_pair, mesh_pile

pytestmark = pytest.mark.gpu


def _solvers(sc, cfg, **kw):
    g_auto, orc = make_pair(sc, cfg, **kw)
    forced = []
    for mode in (0, 1):
        g, _ = make_pair(sc, cfg, gpu=True, **kw)
        g.set_solve_split(mode)
        assert g.solve_split == mode
        forced.append(g)
    return g_auto, forced, orc


def _run(sc, cfg, frames, substeps, iterations, what, **kw):
    g_auto, (g0, g1), orc = _solvers(sc, cfg, **kw)
    assert g_auto.solve_split == -1
    for f in range(frames):
        for s in (g_auto, g0, g1, orc):
            s.step(1.0 / 60.0, substeps, iterations)
        x = orc.get_positions()
        v = orc.get_velocities()
        for name, g in (("auto", g_auto), ("fused", g0), ("split", g1)):
            assert_bitexact(g.get_positions(), x, f"{what} {name} positions frame {f}")
            assert_bitexact(g.get_velocities(), v, f"{what} {name} velocities frame {f}")
            assert g.last_contact_count == orc.last_contact_count, f"{what} {name} contacts frame {f}"
    assert g_auto.solve_split in (0, 1)  # decided after its timed frames
    assert g0.solve_split == 0 and g1.solve_split == 1


def test_split_static_mesh_bitexact():
    sc = mesh_pile(14, hf=32)
    _run(sc, config_for(sc), 7, 5, 1, "mesh")


def test_split_two_iterations_bitexact():
    sc = mesh_pile(12, hf=24)
    _run(sc, config_for(sc), 6, 4, 2, "mesh 2 iterations")


def test_split_with_bodies_bitexact():
    sc = box_scene(n_side=8, boxes=((0.05, 0.04, 0.03), (0.03, 0.03, 0.06)),
                   positions=((0.0, 0.0, 0.2), (0.06, -0.03, 0.32)), hf=24)
    _run(sc, config_for(sc), 7, 5, 1, "bodies")


def test_solve_split_rejects_bad_mode():
    sc = mesh_pile(6, hf=8)
    g, _ = make_pair(sc, config_for(sc), gpu=True)
    with pytest.raises(RuntimeError, match="set_solve_split"):
        g.set_solve_split(2)
