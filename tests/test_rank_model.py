"""The rank algebra of the stable-rank binning, restated on the CPU.

G2P gives a particle that stays in its cell its old rank r_old (< 64) as a
tentative rank and marks the old rank of a particle that leaves in its old
cell's 64-bit leave mask; every other particle (an arrival, a fresh one, or a
stayer ranked 64 or above) counts itself in the cell's arrival counter.
k_scatter then gives a stayer r_old minus the leavers ranked below it, and an
arrival N - A + (its arrival order).  These tests check on random moves that
this yields exactly the ranks 0 .. N-1 in every cell and keeps the stayers'
relative order (the property that makes P2G's gather contiguous).
"""
import numpy as np


def assign_ranks(old_cell, old_rank, new_cell, rng):
    """Ranks in the new cells following the device's rules; arrivals take
    their ranks in a random arrival order."""
    n = len(new_cell)
    stay = (new_cell == old_cell) & (old_rank < 64)
    leave_mask = {}
    for i in np.nonzero((new_cell != old_cell) & (old_rank < 64))[0]:
        leave_mask[old_cell[i]] = leave_mask.get(old_cell[i], 0) | (1 << int(old_rank[i]))
    cells, counts = np.unique(new_cell, return_counts=True)
    N = dict(zip(cells.tolist(), counts.tolist()))
    A = {}
    for i in np.nonzero(~stay)[0]:
        A[new_cell[i]] = A.get(new_cell[i], 0) + 1
    rank = np.empty(n, np.int64)
    for i in np.nonzero(stay)[0]:
        below = leave_mask.get(new_cell[i], 0) & ((1 << int(old_rank[i])) - 1)
        rank[i] = old_rank[i] - bin(below).count("1")
    arrived = {}
    for i in rng.permutation(np.nonzero(~stay)[0]):
        c = new_cell[i]
        rank[i] = N[c] - A[c] + arrived.get(c, 0)
        arrived[c] = arrived.get(c, 0) + 1
    return rank, stay


def initial_ranks(cell, rng):
    rank = np.empty(len(cell), np.int64)
    for c in np.unique(cell):
        idx = np.nonzero(cell == c)[0]
        rank[idx] = rng.permutation(len(idx))
    return rank


def test_ranks_are_a_permutation_and_keep_stayer_order():
    rng = np.random.default_rng(0)
    for ncells, n, p_move in ((50, 2000, 0.05), (8, 3000, 0.2), (3, 500, 0.5), (200, 20000, 0.01)):
        cell = rng.integers(0, ncells, n)
        rank = initial_ranks(cell, rng)
        for _ in range(5):
            move = rng.random(n) < p_move
            new_cell = np.where(move, rng.integers(0, ncells, n), cell)
            new_rank, stay = assign_ranks(cell, rank, new_cell, rng)
            for c in np.unique(new_cell):
                idx = np.nonzero(new_cell == c)[0]
                np.testing.assert_array_equal(np.sort(new_rank[idx]), np.arange(len(idx)))
                s = idx[stay[idx]]
                # stayers keep their relative order and come first
                assert np.all(np.diff(new_rank[s][np.argsort(rank[s])]) > 0)
                if len(s):
                    assert new_rank[s].max() < len(s)
            cell, rank = new_cell, new_rank


def test_cells_beyond_64_particles():
    """Ranks >= 64 are not tracked in the 64-bit masks: such stayers rank
    after the tracked ones, still a permutation."""
    rng = np.random.default_rng(1)
    n = 1000
    cell = rng.integers(0, 4, n)  # ~250 particles per cell
    rank = initial_ranks(cell, rng)
    new_cell = np.where(rng.random(n) < 0.1, rng.integers(0, 4, n), cell)
    new_rank, stay = assign_ranks(cell, rank, new_cell, rng)
    assert stay.sum() > 0 and (rank >= 64).sum() > 0
    for c in range(4):
        idx = np.nonzero(new_cell == c)[0]
        np.testing.assert_array_equal(np.sort(new_rank[idx]), np.arange(len(idx)))
