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
    import scenes
    from vkxpbd import _abi

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


def _noalloc_sort(lib, keys, key_bits, torch, dev):
    n = keys.size
    d_keys = torch.from_numpy(keys.view(np.int32).copy()).to(dev)
    d_out_k = torch.full((n,), -1, dtype=torch.int32, device=dev)
    d_out_v = torch.full((n,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.xpbd_sort_keys_noalloc(C.c_void_p(d_keys.data_ptr()), C.c_void_p(d_out_k.data_ptr()),
                                    C.c_void_p(d_out_v.data_ptr()), n, key_bits, C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return rc, d_out_k.cpu().numpy().view(np.uint32), d_out_v.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [13_824, 1 << 20])
@pytest.mark.parametrize("key_bits", [21, 32])
def test_noalloc_sort_random_keys_stable(n, key_bits):
    """Up to the stated maximum (1,048,576 keys: every look-back word of the array in use) and
    with 32-bit keys (four radix passes, so the first pass writes the scratch pair): sorted
    keys and ids against numpy's stable argsort, twice in a row on different keys."""
    import torch

    from helpers import assert_bitexact
    from vkxpbd import _abi

    lib = _abi.load()
    dev = torch.device("cuda", 0)
    for call in range(2):
        rng = np.random.default_rng(1000 * call + key_bits)
        hi = 1 << key_bits
        # many equal keys as in a hash grid (a few values repeated), so stability matters
        keys = rng.integers(0, min(hi, 4 * n), size=n, dtype=np.uint64)
        if key_bits == 32:
            keys = (keys * 2654435761) % hi  # spread over the whole word
        keys = keys.astype(np.uint32)
        rc, out_k, out_v = _noalloc_sort(lib, keys, key_bits, torch, dev)
        assert rc == 0, lib.xpbd_last_error().decode()
        order = np.argsort(keys, kind="stable").astype(np.uint32)
        assert_bitexact(out_v, order, f"n={n} bits={key_bits} call {call}: ids")
        assert_bitexact(out_k, keys[order], f"n={n} bits={key_bits} call {call}: keys")


def test_noalloc_sort_reports_a_timed_out_wait():
    """A look-back wait that runs out (one tile held back by the test hook, 1 ms limit) makes
    the call fail instead of returning a wrong order; the next call is exact again."""
    import torch

    import vkxpbd
    from helpers import assert_bitexact
    from vkxpbd import _abi

    lib = _abi.load()
    dev = torch.device("cuda", 0)
    keys = np.random.default_rng(5).integers(0, 1 << 21, size=20_000, dtype=np.uint32)
    vkxpbd.debug_lookback_hold(2, 1_000_000)
    try:
        rc, _, _ = _noalloc_sort(lib, keys, 21, torch, dev)
        assert rc != 0
        assert "timed out" in lib.xpbd_last_error().decode()
    finally:
        vkxpbd.debug_lookback_hold(-1)
    rc, out_k, out_v = _noalloc_sort(lib, keys, 21, torch, dev)
    assert rc == 0, lib.xpbd_last_error().decode()
    order = np.argsort(keys, kind="stable").astype(np.uint32)
    assert_bitexact(out_v, order, "ids after the timed-out call")
    assert_bitexact(out_k, keys[order], "keys after the timed-out call")


def test_noalloc_sort_inside_a_cuda_graph_capture():
    """The call recorded into another framework's CUDA graph (torch.cuda.graph): no allocation
    while capturing or replaying, each replay sorts the keys then in the input buffer, and the
    replay's status is read afterwards with xpbd_sort_keys_noalloc_status."""
    import torch

    from helpers import assert_bitexact
    from vkxpbd import _abi

    lib = _abi.load()
    dev = torch.device("cuda", 0)
    n = 50_000
    rng = np.random.default_rng(11)
    d_keys = torch.zeros(n, dtype=torch.int32, device=dev)
    d_out_k = torch.zeros(n, dtype=torch.int32, device=dev)
    d_out_v = torch.zeros(n, dtype=torch.int32, device=dev)

    def call():
        return lib.xpbd_sort_keys_noalloc(C.c_void_p(d_keys.data_ptr()), C.c_void_p(d_out_k.data_ptr()),
                                          C.c_void_p(d_out_v.data_ptr()), n, 21,
                                          C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))

    assert call() == 0, lib.xpbd_last_error().decode()  # first call on the device: outside the capture
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rc = call()
    assert rc == 0, lib.xpbd_last_error().decode()
    allocated = torch.cuda.memory_allocated(dev)
    for rep in range(3):
        keys = rng.integers(0, 1 << 21, size=n, dtype=np.uint32)
        d_keys.copy_(torch.from_numpy(keys.view(np.int32)))
        graph.replay()
        torch.cuda.synchronize(dev)
        assert lib.xpbd_sort_keys_noalloc_status() == 0, lib.xpbd_last_error().decode()
        order = np.argsort(keys, kind="stable").astype(np.uint32)
        assert_bitexact(d_out_v.cpu().numpy().view(np.uint32), order, f"replay {rep}: ids")
        assert_bitexact(d_out_k.cpu().numpy().view(np.uint32), keys[order], f"replay {rep}: keys")
    assert torch.cuda.memory_allocated(dev) == allocated


def test_noalloc_sort_rejects_too_many_keys():
    from vkxpbd import _abi

    lib = _abi.load()
    rc = lib.xpbd_sort_keys_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), (1 << 20) + 1, 21, None)
    assert rc != 0
    assert "at most 1048576" in lib.xpbd_last_error().decode()


def test_noalloc_sort_rejects_overlapping_buffers():
    """The input must not overlap an output: a pass could overwrite keys a later tile still reads."""
    from vkxpbd import _abi

    lib = _abi.load()
    a, b = 1 << 20, 1 << 24
    for keys, out_k, out_v in ((a, a, b), (a, b, a + 64), (a, b, b + 64)):
        rc = lib.xpbd_sort_keys_noalloc(C.c_void_p(keys), C.c_void_p(out_k), C.c_void_p(out_v), 1000, 21, None)
        assert rc != 0
        assert "must not overlap" in lib.xpbd_last_error().decode()
