"""The oracle's multi-segment runs (veb gather_multiple / return_multiple,
veb.cuh:1160-1218, and the run tier of Gallatin::malloc, gallatin.cuh:790-826)
under random request and free orders: runs never overlap, each starts on a
segment boundary, and once everything is freed the segment tree is the fresh
one again."""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import PRODUCT_FIXES, Oracle

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
