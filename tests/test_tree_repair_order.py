"""The event tree's repair order (no GPU).

UpdateCBTRun (src/CBT.c:56-83) repairs a leaf's path incrementally and stops at
the first unchanged node; every repair leaves each node the winner of its two
children (smaller time, ties to the right child).  The engine repairs the
target's path while the partner's fold may still be writing the partner's
time, then gives the partner's path a full repair.  This test checks, on random
trees, that both orders give the reference's tree: the one a full rebuild gives.
"""
import numpy as np


def winner(times, node, f):
    l, r = node[2 * f], node[2 * f + 1]
    return l if times[l] < times[r] else r


def build(times, n, leaf_of):
    node = np.zeros(2 * n, np.int64)
    for a in range(1, n + 1):
        node[leaf_of[a]] = a
    for f in range(n - 1, 0, -1):
        node[f] = winner(times, node, f)
    return node


def update(times, node, leaf_of, a, full=False):
    """UpdateCBTRun: while the node names a it is recomputed; then each node is
    recomputed and the walk stops at the first unchanged one (full: no stop)."""
    f = leaf_of[a] // 2
    while f > 0 and node[f] == a:
        node[f] = winner(times, node, f)
        f //= 2
    while f > 0:
        old = node[f]
        node[f] = winner(times, node, f)
        if node[f] == old and not full:
            return
        f //= 2


def test_overlapped_target_repair_gives_the_reference_tree():
    rng = np.random.default_rng(7)
    for trial in range(3000):
        n = int(rng.integers(2, 70))
        leaf_of = np.zeros(n + 1, np.int64)
        leaf_of[1:] = n + rng.permutation(n)            # leaves n .. 2n-1 in some layout
        times = np.concatenate([[np.inf], rng.integers(0, 6, n).astype(float)])   # many ties
        node = build(times, n, leaf_of)
        t, p = rng.choice(np.arange(1, n + 1), 2, replace=False)
        new_t, new_p = float(rng.integers(0, 6)), float(rng.integers(0, 6))
        # the reference: both events are known, then UpdateCBTRun(t), UpdateCBTRun(p)
        ref_times = times.copy(); ref_times[t] = new_t; ref_times[p] = new_p
        ref = node.copy()
        update(ref_times, ref, leaf_of, t)
        update(ref_times, ref, leaf_of, p)
        # the engine: t repaired while p still holds its old time, then p in full
        eng_times = times.copy(); eng_times[t] = new_t
        eng = node.copy()
        update(eng_times, eng, leaf_of, t)
        eng_times[p] = new_p
        update(eng_times, eng, leaf_of, p, full=True)
        rebuilt = build(ref_times, n, leaf_of)
        assert np.array_equal(ref, rebuilt), trial
        assert np.array_equal(eng, rebuilt), trial


class Racy:
    """Leaf times where p's entry reads old or new at random (a concurrent write)."""
    def __init__(self, times, p, new_p, rng):
        self.t, self.p, self.new_p, self.rng = times, p, new_p, rng

    def __getitem__(self, a):
        if a == self.p and self.rng.integers(0, 2):
            return self.new_p
        return self.t[a]


def test_repair_with_the_partner_time_read_mid_write():
    rng = np.random.default_rng(11)
    for trial in range(3000):
        n = int(rng.integers(2, 70))
        leaf_of = np.zeros(n + 1, np.int64)
        leaf_of[1:] = n + rng.permutation(n)
        times = np.concatenate([[np.inf], rng.integers(0, 6, n).astype(float)])
        node = build(times, n, leaf_of)
        t, p = rng.choice(np.arange(1, n + 1), 2, replace=False)
        new_t, new_p = float(rng.integers(0, 6)), float(rng.integers(0, 6))
        final = times.copy(); final[t] = new_t; final[p] = new_p
        racy_times = times.copy(); racy_times[t] = new_t
        eng = node.copy()
        update(Racy(racy_times, p, new_p, rng), eng, leaf_of, t)
        update(final, eng, leaf_of, p, full=True)
        assert np.array_equal(eng, build(final, n, leaf_of)), trial

