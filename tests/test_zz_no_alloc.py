"""xpbd_sort_keys_noalloc: the allocation-free sort, for callers that cannot
allocate device memory while they run (work captured into another framework's
CUDA graph, plugins inside an application with its own device memory pool,
real-time loops without allocator calls). It must give exactly the hash-grid
sort of the regular solver step (xpbd_step + xpbd_get_sorted_cells /
xpbd_get_sorted_point_ids), call after call, although its scratch array is
shared and keeps the previous call's contents.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver_sorted_keys(solver):
    cells = solver.get_sorted_cells()
    ids = solver.get_sorted_point_ids()
    keys = np.empty_like(cells)
    keys[ids] = cells  # the unsorted per-particle cell keys the step sorted
    return keys, cells, ids


def test_noalloc_sort_matches_solver_sort_twice():
    import torch

    from helpers import assert_bitexact, config_for, make_pair
    from vkxpbd import _abi, scenes

    lib = _abi.load()
    sc = scenes.pile(dims=(24, 24, 24))
    cfg = config_for(sc)
    g, _ = make_pair(sc, cfg)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):  # two calls in a row, on different key sets
        g.step(1.0 / 60.0, 3, 1)
        keys, ref_cells, ref_ids = _solver_sorted_keys(g)
        n = keys.size
        d_keys = torch.from_numpy(keys.view(np.int32).copy()).to(dev)
        d_out_k = torch.full((n,), -1, dtype=torch.int32, device=dev)
        d_out_v = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rc = lib.xpbd_sort_keys_noalloc(C.c_void_p(d_keys.data_ptr()), C.c_void_p(d_out_k.data_ptr()),
                                        C.c_void_p(d_out_v.data_ptr()), n, 21, C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.xpbd_last_error().decode()
        torch.cuda.synchronize(dev)
        out_k = d_out_k.cpu().numpy().view(np.uint32)
        out_v = d_out_v.cpu().numpy().view(np.uint32)
        assert_bitexact(out_k, ref_cells, f"call {call}: sorted keys")
        assert_bitexact(out_v, ref_ids, f"call {call}: sorted ids")


def test_noalloc_sort_rejects_too_many_keys():
    from vkxpbd import _abi

    lib = _abi.load()
    rc = lib.xpbd_sort_keys_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), (1 << 20) + 1, 21, None)
    assert rc != 0
    assert "at most 1048576" in lib.xpbd_last_error().decode()
