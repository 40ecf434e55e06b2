"""GPU LBVH build and refit (k_bvh.cu) against the reference builder's golden
output (tests/golden/bvh_golden.npz, made by the reference's own
mesh_lbvh.h / mesh_bvh.h) and against the oracle on the bench heightfield."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import assert_bitexact

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bvh_golden.npz")


def _names():
    g = np.load(GOLDEN)
    return sorted({k.split("/")[0] for k in g.files})


def _solver_with(meshes):
    import vkxpbd

    cfg = vkxpbd.SolverConfig()
    s = vkxpbd.XpbdSolver()
    s.init(cfg, 1)
    for v, t in meshes:
        s.add_mesh(v, t)
    s.finalize_meshes()
    return s


@pytest.mark.parametrize("name", _names())
def test_gpu_bvh_matches_reference_golden(name):
    g = np.load(GOLDEN)
    s = _solver_with([(g[f"{name}/verts"], g[f"{name}/tris"])])
    lo = np.asarray(s.get_mesh_bvh_lowers(0), np.float32).reshape(-1, 4)
    hi = np.asarray(s.get_mesh_bvh_uppers(0), np.float32).reshape(-1, 4)
    assert_bitexact(lo, g[f"{name}/lowers"].reshape(-1, 4), f"{name} lowers")
    assert_bitexact(hi, g[f"{name}/uppers"].reshape(-1, 4), f"{name} uppers")
    s.update_mesh(0, g[f"{name}/verts_moved"])
    lo = np.asarray(s.get_mesh_bvh_lowers(0), np.float32).reshape(-1, 4)
    hi = np.asarray(s.get_mesh_bvh_uppers(0), np.float32).reshape(-1, 4)
    assert_bitexact(lo, g[f"{name}/refit_lowers"].reshape(-1, 4), f"{name} refit lowers")
    assert_bitexact(hi, g[f"{name}/refit_uppers"].reshape(-1, 4), f"{name} refit uppers")


def test_gpu_bvh_of_several_meshes_and_bench_heightfield():
    import scenes

    hv, ht = scenes.heightfield(256)
    bv, bt = scenes.box_mesh((0.1, 0.2, 0.05), center=(0.1, 0.0, 0.3), quat_xyzw=(0.2, 0.1, 0.0, 0.97))
    s = _solver_with([(bv, bt), (hv, ht)])
    for i, (v, t) in enumerate([(bv, bt), (hv, ht)]):
        lo, hi, pr, root = O.bvh_build(v, t)
        assert_bitexact(np.asarray(s.get_mesh_bvh_lowers(i), np.float32).reshape(-1, 4), lo.reshape(-1, 4),
                        f"mesh {i} lowers")
        assert_bitexact(np.asarray(s.get_mesh_bvh_uppers(i), np.float32).reshape(-1, 4), hi.reshape(-1, 4),
                        f"mesh {i} uppers")
