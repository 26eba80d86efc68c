"""Random request/free traces over every size tier (slices, 4 KiB-slice runs,
whole blocks, segment runs) through the oracle with the product's fixes.

Along the way each vEB tree (the segment tree and every per-class sub-tree,
veb.cuh) keeps its summary exact: a summary bit is set exactly when the word
below it is non-empty, which a serial trace must preserve (insert climbs from
an empty word, remove from a word it empties, gather and return of a run
update the words they touch).  Live requests never overlap and slices sit on
their class boundary.  Freeing everything and trimming gives back a fresh
allocator's trees.  In the reference's mode (FIX_RUN_RETURN_SUMMARY off) some
of these seeds leave a word unlisted."""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import FIX_RUN_RETURN_SUMMARY, PRODUCT_FIXES, Oracle

SEG = 16 << 20
TREE_FIELDS = ["seg_tree_words", "sub_tree_words", "tree_ids", "slots", "free_counters"]


def layer_words(universe):
    """Words per layer, top first, as the tree lays them out (veb.cuh:541-576)."""
    layers = (universe.bit_length() - 1) // 6 + 1
    out, u = [], universe
    for _ in range(layers):
        u = (u - 1) // 64 + 1
        out.insert(0, u)
    return out


def unlisted(words, universe):
    """(layer, word) of the first summary bit that disagrees with its word."""
    sizes = layer_words(universe)
    offs = np.cumsum([0] + sizes)
    assert offs[-1] == len(words)
    for i in range(len(sizes) - 1):
        up, lo = words[offs[i]:offs[i + 1]], words[offs[i + 1]:offs[i + 2]]
        for k in range(len(lo)):
            if bool(int(up[k // 64]) >> (k % 64) & 1) != (int(lo[k]) != 0):
                return i + 1, k
    return None


def summaries_exact(o):
    d = o.dims()
    sv = o.export()
    if unlisted(sv.seg_tree_words, d.num_segments):
        return False
    W = d.veb_words
    return all(unlisted(sv.sub_tree_words[t * W:(t + 1) * W], d.num_segments) is None
               for t in range(d.num_trees))


def run_trace(seed, fixes, nops=1500, nbytes=None, max_run=8, every=10):
    rng = np.random.default_rng(seed)
    nbytes = nbytes or [2 << 30, 4 << 30][seed % 2]
    o = Oracle(nbytes, 42, fixes=fixes, spares=bool(seed & 2))
    fresh = o.export()
    live = {}
    for i in range(nops):
        if live and rng.random() < 0.45:
            off = list(live)[int(rng.integers(len(live)))]
            o.free(off)
            del live[off]
            continue
        t = rng.random()
        if t < 0.4:
            size = int(rng.integers(1, 4097))
        elif t < 0.8:
            size = int(rng.integers(32769, SEG + 1))
        else:
            size = int(rng.integers(SEG + 1, max_run * SEG))
        off = o.malloc(size, smid=int(rng.integers(4)), tid=i)
        if off != FAIL:
            assert off not in live and off + size <= o.arena_bytes
            if size <= 4096:
                assert off % max(16, 1 << (size - 1).bit_length()) == 0
            live[off] = size
        if i % every == 0:
            if not summaries_exact(o):
                return False
            spans = sorted(live.items())
            assert all(a + n <= b for (a, n), (b, _) in zip(spans, spans[1:]))
    for off in list(live):
        o.free(off)
    o.trim()
    assert o.export().diff(fresh, fields=TREE_FIELDS) == []
    return summaries_exact(o)


@pytest.mark.parametrize("seed", range(24))
def test_random_tiers_keep_summaries_exact_and_drain_to_fresh_trees(seed):
    assert run_trace(seed, PRODUCT_FIXES)


def test_the_reference_rule_leaves_words_unlisted():
    """Seeds 3, 5, 9, 15, 22 and 23 of the same traces, with the reference's
    return rule, list a non-empty word in no summary at some point."""
    fixes = PRODUCT_FIXES & ~FIX_RUN_RETURN_SUMMARY
    assert [s for s in range(24) if not run_trace(s, fixes)] == [3, 5, 9, 15, 22, 23]


@pytest.mark.parametrize("fixes,exact", [(PRODUCT_FIXES, True),
                                         (PRODUCT_FIXES & ~FIX_RUN_RETURN_SUMMARY, False)],
                         ids=["product", "reference"])
def test_three_layer_trees(fixes, exact):
    """64 GiB = 4,096 segments: the trees have three layers, so claims and
    returns of runs of up to 200 segments update two summary layers."""
    assert run_trace(0, fixes, nops=2500, nbytes=64 << 30, max_run=200, every=250) == exact


def tier_trace(seed, nops=1500):
    """A serial trace (malloc sizes; 1<<63 | index frees of earlier mallocs not
    yet freed) with the tier mix above, fixed before any replay."""
    rng = np.random.default_rng(seed)
    ops, open_ = [], []
    for i in range(nops):
        if open_ and rng.random() < 0.45:
            ops.append((1 << 63) | open_.pop(int(rng.integers(len(open_)))))
            continue
        t = rng.random()
        if t < 0.4:
            ops.append(int(rng.integers(1, 4097)))
        elif t < 0.8:
            ops.append(int(rng.integers(32769, SEG + 1)))
        else:
            ops.append(int(rng.integers(SEG + 1, 8 * SEG)))
        open_.append(i)
    return np.array(ops, dtype=np.uint64)


@pytest.mark.parametrize("seed", [3, 9])
def test_tier_traces_replay_with_exact_summaries(seed):
    o = Oracle([2 << 30, 4 << 30][seed % 2], 42, fixes=PRODUCT_FIXES)
    out = o.replay(tier_trace(seed))
    assert (out != FAIL).sum() > 500
    assert summaries_exact(o)


@pytest.mark.parametrize("seed", range(8))
def test_trims_inside_a_trace_keep_live_requests_apart(seed):
    """Trim at random points (a full arena leaves the slots it cannot fill
    empty), one slot per SM or the reference's counts, with or without spare
    blocks: live requests never overlap, summaries stay exact, and freeing
    everything then trimming gives back the fresh trees."""
    rng = np.random.default_rng(seed)
    o = Oracle([1 << 30, 2 << 30][seed % 2], 42, spares=bool(seed & 2),
               pinned_first=[128, 0][(seed >> 2) & 1])
    fresh = o.export()
    live = {}
    for i in range(2000):
        r = rng.random()
        if r < 0.01:
            try:
                o.trim()
            except RuntimeError:
                pass                                   # arena full: some slots stay empty
            continue
        if live and r < 0.45:
            off = list(live)[int(rng.integers(len(live)))]
            o.free(off)
            del live[off]
            continue
        size = int(rng.choice([rng.integers(1, 4097), rng.integers(4097, 32769),
                               rng.integers(32769, SEG + 1), rng.integers(SEG + 1, 5 * SEG)],
                              p=[0.6, 0.15, 0.2, 0.05]))
        off = o.malloc(size, smid=int(rng.integers(152)), tid=i)
        if off != FAIL:
            assert off not in live
            live[off] = size
        if i % 50 == 0:
            spans = sorted(live.items())
            assert all(a + n <= b for (a, n), (b, _) in zip(spans, spans[1:]))
            assert summaries_exact(o)
    for off in list(live):
        o.free(off)
    o.trim()
    assert o.export().diff(fresh, fields=TREE_FIELDS) == []
