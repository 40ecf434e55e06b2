"""Generates tests/golden/bvh_golden.npz from the reference's own BVH code.

Runs only where oracle/_ref/libref_bvh.so exists (built in place from the
reference checkout by `make -C oracle ref`). For each seeded mesh it stores the
inputs and the reference's MeshBvh::build output (src/mesh_bvh.h:40-69 ->
src/mesh_lbvh.h:49-223), the node halves after a MeshBvh::refit
(src/mesh_bvh.h:142-181) with displaced vertices, and a brute-force closest
point query (src/mesh_bvh.h:296-321). Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "newton-xpbd-vulkan_gb300")]

import oracle as O  # noqa: E402
import scenes  # noqa: E402


def meshes():
    rng = np.random.default_rng(7)
    out = {}
    out["hf16"] = scenes.heightfield(16, extent=0.4, amplitude=0.02)
    out["hf48"] = scenes.heightfield(48)
    out["box"] = scenes.box_mesh((0.05, 0.08, 0.03), (0.1, -0.2, 0.3), (0.1, 0.2, 0.3, 0.9273618))
    for n in (1, 2, 3, 7, 33, 257):
        out[f"soup{n}"] = (rng.random((3 * n, 3)).astype(np.float32), np.arange(3 * n, dtype=np.uint32).reshape(-1, 3))
    pts = np.repeat(rng.random((6, 3)).astype(np.float32), 20, axis=0)
    out["ties"] = (pts, rng.integers(0, pts.shape[0], (200, 3)).astype(np.uint32))
    return out


def main():
    ref = O.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_bvh.so not built (make -C oracle ref REF=<reference checkout>)")
    rng = np.random.default_rng(11)
    blob = {}
    for name, (v, t) in meshes().items():
        lo, hi, pr, root = O.ref_bvh_build(ref, v, t)
        v2 = (v + rng.normal(0, 0.01, v.shape)).astype(np.float32)
        rlo, rhi = O.ref_bvh_build_refit(ref, v, v2, t)
        blob[f"{name}/verts"] = v
        blob[f"{name}/tris"] = t
        blob[f"{name}/lowers"] = lo
        blob[f"{name}/uppers"] = hi
        blob[f"{name}/prims"] = pr
        blob[f"{name}/root"] = np.array([root], np.uint32)
        blob[f"{name}/verts_moved"] = v2
        blob[f"{name}/refit_lowers"] = rlo
        blob[f"{name}/refit_uppers"] = rhi
    np.savez_compressed(os.path.join(HERE, "bvh_golden.npz"), **blob)
    print("wrote", os.path.join(HERE, "bvh_golden.npz"), len(blob), "arrays")


if __name__ == "__main__":
    main()
