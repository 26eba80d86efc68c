"""The oracle's multi-segment runs (veb gather_multiple / return_multiple,
veb.cuh:1160-1218, and the run tier of Gallatin::malloc, gallatin.cuh:790-826)
under random request and free orders: runs never overlap, each starts on a
segment boundary, and once everything is freed the segment tree is the fresh
one again."""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import FIX_RUN_RETURN_SUMMARY, PRODUCT_FIXES, Oracle

SEG = 16 << 20


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_runs_are_disjoint_and_drain_to_the_fresh_tree(seed):
    rng = np.random.default_rng(seed)
    o = Oracle(1 << 30, 42, fixes=PRODUCT_FIXES, boot=False)   # 64 segments, no pinned blocks
    fresh = o.export()
    live = {}
    for _ in range(400):
        if live and rng.random() < 0.45:
            off = list(live)[int(rng.integers(len(live)))]
            o.free(off)
            del live[off]
            continue
        k = int(rng.integers(2, 9))                               # 2..8 segments
        size = k * SEG - int(rng.integers(0, SEG // 2))
        off = o.malloc(size)
        if off == FAIL:
            continue
        assert off % SEG == 0
        live[off] = k
        spans = sorted((a, a + n * SEG) for a, n in live.items())
        assert all(e0 <= s1 for (_, e0), (s1, _) in zip(spans, spans[1:]))
        assert spans[-1][1] <= o.arena_bytes()
    for off in list(live):
        o.free(off)
    assert o.export().diff(fresh, fields=["seg_tree_words", "tree_ids"]) == []


def test_a_run_larger_than_the_arena_fails_cleanly():
    o = Oracle(1 << 30, 42, fixes=PRODUCT_FIXES, boot=False)
    fresh = o.export()
    assert o.malloc(65 * SEG) == FAIL
    assert o.export().diff(fresh) == []


# A run that still needs more than the words below it: the reference steps to
# bottom-layer word -1 (veb.cuh:382-410); the product fails and gives back what
# it took.  On 128 segments: 65-115 and 119-127 in use, the request of 84
# takes segment 64 and all of word 0 and would need 19 more below word 0.
RUN_BELOW_ARENA = [("m", 85), ("f", 0), ("m", 64), ("f", 1), ("m", 9), ("m", 3), ("m", 51),
                   ("m", 61), ("m", 56), ("m", 93), ("f", 3), ("f", 5)]


def replay_runs(o, steps):
    got = []
    for op, x in steps:
        if op == "m":
            got.append(o.malloc(x * SEG))
        else:
            o.free(got[x])
    return got


def test_a_run_below_the_arena_fails_and_gives_back_what_it_took():
    o = Oracle(2 << 30, 42, fixes=PRODUCT_FIXES, boot=False)
    got = replay_runs(o, RUN_BELOW_ARENA)
    assert [g // SEG if g != FAIL else -1 for g in got] == [43, 64, 119, 116, 65, 4, -1, -1]
    before = o.export()
    assert o.malloc(84 * SEG) == FAIL
    assert o.export().diff(before) == []
    # word 0 is whole again: a run of 64 takes segment 64 and the top 63 of it
    assert o.malloc(64 * SEG) == 1 * SEG


# Returning a run lists a bottom word in the summary only when the word is then
# full (maybe_return_layer_bits, veb.cuh:1128-1154).  On 128 segments a run of
# 34 takes 94-127 and a run of 36 takes 58-93, emptying word 1; freeing the
# second gives 64-93 back to word 1, which is not full, so the reference leaves
# it unlisted and the single-item searches never see those 30 segments.
HIDDEN_BY_RETURN = [("m", 34), ("m", 36), ("f", 1)]


def runs_to_ops(steps):
    """The serial trace (malloc sizes, 1<<63 | index frees) of a run list."""
    ops, idx = [], []
    for op, x in steps:
        if op == "m":
            idx.append(len(ops))
            ops.append(x * SEG)
        else:
            ops.append((1 << 63) | idx[x])
    return np.array(ops, dtype=np.uint64), idx


def summary_lists_every_nonempty_word(sv):
    top, bottom = int(sv.seg_tree_words[0]), sv.seg_tree_words[1:3]
    return all(bool(top >> k & 1) == (int(w) != 0) for k, w in enumerate(bottom))


@pytest.mark.parametrize("fixes,reachable", [
    (PRODUCT_FIXES & ~FIX_RUN_RETURN_SUMMARY, 64),   # the reference: 30 segments unreachable
    (PRODUCT_FIXES, 94),
], ids=["reference", "product"])
def test_a_returned_run_lists_every_word_it_refills(fixes, reachable):
    o = Oracle(2 << 30, 42, fixes=fixes, boot=False)
    got = replay_runs(o, HIDDEN_BY_RETURN)
    assert [g // SEG for g in got] == [94, 58]
    assert summary_lists_every_nonempty_word(o.export()) == (fixes == PRODUCT_FIXES)
    singles = []
    while (x := o.malloc(SEG)) != FAIL:
        singles.append(x // SEG)
    assert len(singles) == reachable and len(set(singles)) == reachable
    assert not set(singles) & set(range(94, 128))
