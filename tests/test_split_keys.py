"""Split hash-grid keys (CPU property test of the argument the solve relies on).

The reference keys a particle by its cell on a 128^3 grid that wraps every 128 cells
(grid_cell_indices.comp:17-25); one-scene solvers here sort by that key plus bit 7 of each
axis' unwrapped cell coordinate. The neighbour loop (solve_particle_particle_contacts.comp:
126-157) visits, for each cell of a particle's neighbourhood, the particles of that key's
range in sorted order and keeps those within reach. With a stable sort from particle order,
both layouts must give every particle the same accepted neighbours in the same order.
This restates the key functions in numpy (the same integer arithmetic as the kernels) and
checks that on clusters placed 128 and 256 cells apart, across the 128-cell boundary and
at clamped coordinates.
"""
import numpy as np

ORIGIN = 1 << 20


def _cells(x, inv):
    return np.floor(x.astype(np.float32) * np.float32(inv)).astype(np.int64)


def _key(g, split):
    """g: unwrapped cell coordinates + origin, clamped at 0 (the kernels' imax0)."""
    g = np.maximum(g, 0)
    k = (g[..., 2] % 128) * 128 * 128 + (g[..., 1] % 128) * 128 + (g[..., 0] % 128)
    if split:
        k = k | (((g[..., 0] >> 7) & 1) << 21) | (((g[..., 1] >> 7) & 1) << 22) | (((g[..., 2] >> 7) & 1) << 23)
    return k


def _neighbours(x, r, inv, split):
    n = x.shape[0]
    keys = _key(_cells(x, inv) + ORIGIN, split)
    order = np.argsort(keys, kind="stable")  # ties in particle order
    skeys = keys[order]
    out = []
    for i in range(n):
        R = r + r  # radius + max radius, no cohesion
        lo = _cells(x[i] - R, inv)
        hi = _cells(x[i] + R, inv)
        acc = []
        for cz in range(lo[2], hi[2] + 1):
            for cy in range(lo[1], hi[1] + 1):
                for cx in range(lo[0], hi[0] + 1):
                    k = _key(np.array([cx, cy, cz]) + ORIGIN, split)
                    a, b = np.searchsorted(skeys, k, "left"), np.searchsorted(skeys, k, "right")
                    for j in order[a:b]:
                        if j == i:
                            continue
                        d = x[i].astype(np.float64) - x[j]
                        if np.all(np.abs(d) <= R) and np.dot(d, d) < (2 * r) ** 2:
                            acc.append(int(j))
        out.append(acc)
    return out


def _scene(seed=3):
    rng = np.random.default_rng(seed)
    cell = 0.02
    base = rng.uniform(0.0, 0.12, size=(60, 3))
    shifts = [(0, 0, 0), (128 * cell, 0, 0), (256 * cell, 0, 0), (0, 128 * cell, 0), (0, 0, 128 * cell),
              (128 * cell - 0.05, 0.3, 0), (-128 * cell - 0.03, 0, 0)]
    x = np.concatenate([base + np.asarray(s) for s in shifts])
    far = np.array([[-3.0e4, 0.0, 0.0], [-3.0e4, 0.01, 0.0], [-3.0e4, 0.0, 0.015]])  # clamped to cell 0 in x
    return np.concatenate([x, far]).astype(np.float32), cell


def test_split_keys_keep_accepted_neighbours_and_order():
    x, cell = _scene()
    r = 0.012
    ref = _neighbours(x, r, 1.0 / cell, split=False)
    spl = _neighbours(x, r, 1.0 / cell, split=True)
    assert sum(len(a) for a in ref) > 100
    assert ref == spl


def test_split_keys_low_bits_are_the_reference_key():
    x, cell = _scene(seed=8)
    g = _cells(x, 1.0 / cell) + ORIGIN
    assert np.array_equal(_key(g, True) & ((1 << 21) - 1), _key(g, False))
    # clusters 128 cells apart share reference keys but not split keys
    a = np.array([[5, 7, 9]]) + ORIGIN
    b = a + np.array([[128, 0, 0]])
    assert _key(a, False)[0] == _key(b, False)[0] and _key(a, True)[0] != _key(b, True)[0]
