"""The incremental binning's position formulas (csrc/mpm_binning.cuh, k_keys_moved ..
k_merge_unmoved) restated in numpy and checked against a stable sort by block, on the CPU.

The slots arrive with previous blocks p (non-decreasing) and new keys k. With moved(i) =
(block(k_i) != p_i), nm(x) = #unmoved slots below x, and for a moved slot q with new block
b the anchor = the first slot whose previous block is >= b (b > p_q) or > b (b < p_q):
  moved slot, j-th in (b, q) order  -> j + nm(anchor)
  unmoved slot i                    -> nm(i) + #{moved j : nm(anchor_j) <= nm(i)}
These must be the positions of the stable sort by block for ANY non-decreasing p (stale
previous keys cost speed, not exactness), with blocks compared as the radix passes see
them, (key >> 6) & umask, and removed particles (key 0xFFFFFFFF) last.
"""
import numpy as np
import pytest

SENTINEL = np.uint32(0xFFFFFFFF)


def block(keys, umask):
    return (keys.astype(np.uint64) >> 6) & np.uint64(umask)


def merge_positions(prev_keys, new_keys, umask):
    """Destination of every slot, by the kernels' formulas."""
    n = len(new_keys)
    p = block(prev_keys, umask)
    b = block(new_keys, umask)
    moved = b != p
    mb = np.concatenate([[0], np.cumsum(moved)])          # moved slots below x, x in [0, n]
    nm = np.arange(n + 1) - mb
    q = np.flatnonzero(moved)
    # anchors: first slot with p >= b (moved up) or p > b (moved down)
    up = b[q] > p[q]
    anchor = np.where(up, np.searchsorted(p, b[q], side="left"), np.searchsorted(p, b[q], side="right"))
    # the galloping search only looks above q when moving up and at or below q when moving down
    assert np.all(anchor[up] > q[up]) and np.all(anchor[~up] <= q[~up])
    R = nm[anchor]
    order = np.argsort(b[q], kind="stable")                # moved slots in (b, q) order
    dest = np.empty(n, np.int64)
    dest[q[order]] = np.arange(len(q)) + R[order]
    Rs = np.sort(R)
    assert np.array_equal(Rs, R[order]), "R is non-decreasing in (b, q) order"
    u = np.flatnonzero(~moved)
    dest[u] = nm[u] + np.searchsorted(Rs, nm[u], side="right")
    return dest


def check(prev_keys, new_keys, umask):
    dest = merge_positions(prev_keys, new_keys, umask)
    assert np.array_equal(np.sort(dest), np.arange(len(new_keys))), "not a permutation"
    perm = np.empty_like(dest)
    perm[dest] = np.arange(len(dest))
    want = np.argsort(block(new_keys, umask), kind="stable")
    assert np.array_equal(perm, want)
    return perm


def keys_of(blocks, rng):
    return ((blocks.astype(np.uint64) << 6) | rng.integers(0, 64, len(blocks)).astype(np.uint64)).astype(np.uint32)


@pytest.mark.parametrize("seed", range(6))
def test_merge_equals_stable_sort_after_small_moves(seed):
    rng = np.random.default_rng(seed)
    n, nb = 5000, 300
    prev_blocks = np.sort(rng.integers(0, nb, n))
    prev = keys_of(prev_blocks, rng)
    new_blocks = prev_blocks.copy()
    mv = rng.random(n) < 0.03
    new_blocks[mv] += rng.choice([-17, -1, 1, 17], mv.sum())
    new_blocks = np.clip(new_blocks, 0, nb - 1)
    new = keys_of(new_blocks, rng)
    gone = rng.random(n) < 0.01                             # removed this substep
    new[gone] = SENTINEL
    check(prev, new, 0xFFFF)


def test_merge_with_removed_particles_already_last():
    rng = np.random.default_rng(7)
    n = 3000
    prev_blocks = np.sort(rng.integers(0, 100, n - 200))
    prev = np.concatenate([keys_of(prev_blocks, rng), np.full(200, SENTINEL, np.uint32)])
    new = prev.copy()
    new[rng.choice(n - 200, 50, replace=False)] = SENTINEL
    check(prev, new, 0xFFFF)


@pytest.mark.parametrize("prev_kind", ["all_ones", "zeros", "stale"])
def test_merge_is_exact_for_any_non_decreasing_previous_keys(prev_kind):
    """The first grid build (all ones), a constant, or the keys of an unrelated order."""
    rng = np.random.default_rng(11)
    n = 4000
    new = keys_of(rng.integers(0, 500, n), rng)
    new[rng.random(n) < 0.02] = SENTINEL
    if prev_kind == "all_ones":
        prev = np.full(n, SENTINEL, np.uint32)
    elif prev_kind == "zeros":
        prev = np.zeros(n, np.uint32)
    else:
        prev = np.sort(keys_of(rng.integers(0, 500, n), rng))
    check(prev, new, 0xFFFF)


def test_blocks_compared_as_the_radix_passes_see_them():
    """With two 8-bit passes only block bits 0-15 are sorted on; the merge uses the same
    truncation, so both agree on keys whose high block bits differ."""
    rng = np.random.default_rng(3)
    n = 2000
    prev_blocks = np.sort(rng.integers(0, 1 << 16, n))
    new_blocks = prev_blocks + (rng.integers(0, 4, n) << 16)   # differ only above bit 15
    check(keys_of(prev_blocks, rng), keys_of(new_blocks, rng), 0xFFFF)
