"""The reference defects the product fixes, shown on the CPU oracle.

Leftover credit (block.cuh:267-281): a malloc whose run of slices crosses the
end of its block credits the slices it could not use to the block's free
counter with a plain atomicAdd, on the comment's premise that some slice of the
block is still live.  When every other slice has been freed, that credit is
the one that completes the block, and the reference never returns it.
"""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import (FIX_GATHER_EXIT_ROLLBACK, FIX_LEFTOVER_COMPLETES, PRODUCT_FIXES,
                           Oracle, gen_leftover_trace, gen_log_trace, gen_serial_trace)

# (max_size, slice size of the largest class): one block per segment, and four
GEOMETRIES = [(4096, 4096), (1024, 1024)]


@pytest.mark.parametrize("max_size,slice_size", GEOMETRIES)
def test_leftover_credit_leaks_block_in_reference(max_size, slice_size):
    ops = gen_leftover_trace(slice_size)
    ref = Oracle(1 << 30, 5, max_size=max_size, fixes=FIX_GATHER_EXIT_ROLLBACK)
    out = ref.replay(ops)
    assert (out[:4095] != FAIL).all() and out[-2] != FAIL
    fc = ref.export().free_counters
    leaked = np.flatnonzero(fc == 4096)
    assert len(leaked) == 1, "the reference keeps the completed block's count at 4096"


@pytest.mark.parametrize("max_size,slice_size", GEOMETRIES)
def test_leftover_credit_returns_block_with_fix(max_size, slice_size):
    ops = gen_leftover_trace(slice_size)
    ref = Oracle(1 << 30, 5, max_size=max_size, fixes=FIX_GATHER_EXIT_ROLLBACK)
    fixed = Oracle(1 << 30, 5, max_size=max_size, fixes=PRODUCT_FIXES)
    out_ref, out_fix = ref.replay(ops), fixed.replay(ops)
    assert (out_fix[:4095] == out_ref[:4095]).all()
    assert out_fix[-2] != FAIL
    sv_ref, sv_fix = ref.export(), fixed.export()
    assert (sv_fix.free_counters < 4096).all()
    # the completed block went back to its segment: one more ring entry (or the
    # whole segment released) than in the reference
    assert sv_fix.diff(sv_ref) != []
    assert PRODUCT_FIXES & FIX_LEFTOVER_COMPLETES


# ---- trim: with nothing live, the trees, segment classes, slots and free
# counters return to those of a fresh allocator (an addition of the product)

TREE_FIELDS = ["seg_tree_words", "sub_tree_words", "tree_ids", "slots", "free_counters"]


def free_everything(ops):
    """The trace followed by a free of every allocation it leaves live."""
    live = set()
    for i, op in enumerate(ops):
        if int(op) >> 63:
            live.discard(int(op) & ~(1 << 63))
        else:
            live.add(i)
    tail = np.array([(1 << 63) | i for i in sorted(live)], dtype=np.uint64)
    return np.concatenate([np.asarray(ops, dtype=np.uint64), tail])


@pytest.mark.parametrize("mk,nbytes", [
    (lambda: gen_serial_trace(101, 20000, 55, 16, 256), 2 << 30),
    (lambda: gen_log_trace(404, 4000, 55, 4, 26), 16 << 30),
])
@pytest.mark.parametrize("spares", [False, True], ids=["", "spares"])
def test_trim_after_freeing_everything_restores_fresh_trees(mk, nbytes, spares):
    """With spare blocks (the product's gal_config.spare_blocks) trim retires
    the spares first, so the same fresh state comes back."""
    o = Oracle(nbytes, 42, spares=spares)
    fresh = o.export()
    o.replay(free_everything(mk()))
    assert o.export().diff(fresh, fields=TREE_FIELDS) != []  # pinned blocks still partly used
    o.trim()
    assert o.export().diff(fresh, fields=TREE_FIELDS) == []


def test_trim_keeps_live_allocations_out_of_reach():
    """A pinned block with live slices is retired, not reused: after trim the
    slots hold other blocks, and freeing the live slices later completes it."""
    ops = gen_serial_trace(7, 4096, 60, 16, 256)
    o = Oracle(2 << 30, 42)
    out = o.replay(ops)
    live_blocks = {int(x) // 4096 for x, op in zip(out, ops) if not int(op) >> 63 and int(x) != FAIL}
    before = o.export()
    o.trim()
    after = o.export()
    assert not (set(after.slots.tolist()) & set(before.slots.tolist()) & live_blocks)


def test_trim_on_a_full_arena_tries_every_slot():
    """Boot and trim try every pinned slot even after one finds no block, as
    the reference's one-thread boot does (gallatin.cuh:196-221): on a full
    arena trim reports the failure, the slots it could not fill stay empty,
    and once everything is freed another trim gives back the fresh trees."""
    o = Oracle(1 << 30, 42)
    fresh = o.export()
    # a live slice in every pinned slot, so trim retires blocks it cannot
    # return, then whole 1 MiB blocks until no segment is left
    live = [o.malloc(16 << t, smid=i) for t in range(9) for i in range(128)]
    assert FAIL not in live
    while (x := o.malloc(1 << 20)) != FAIL:
        live.append(x)
    with pytest.raises(RuntimeError, match=r"trim failed \(-2\)"):
        o.trim()
    empty = int((o.export().slots == -1).sum())          # no block
    assert 0 < empty < len(fresh.slots)
    for x in live:
        o.free(x)
    o.trim()
    assert o.export().diff(fresh, fields=TREE_FIELDS) == []


def test_failed_run_search_marks_in_use_segments_free_in_reference():
    """veb.cuh:447: when no run is found, the reference's search sets the low
    bits of the segment tree's first word that its last try had taken from
    another word, although that try already gave them back.  On 128 segments:
    segment 0 holds a whole block, a run of 63 takes 65-127, and a run of 65
    fails after trying segment 64 with the top of word 0 -- the reference then
    lists segment 0 as free while it is in use (its next claim would trap,
    gallatin.cuh:1488); the product leaves the tree as it was."""
    from gallatin_gb300._abi import FAIL
    from oracle.oracle import FIX_GATHER_EXIT_ROLLBACK, PRODUCT_FIXES, Oracle
    seg = 16 << 20
    free_bit0 = {}
    for name, fixes in (("reference", PRODUCT_FIXES & ~FIX_GATHER_EXIT_ROLLBACK), ("product", PRODUCT_FIXES)):
        o = Oracle(2 << 30, 42, fixes=fixes, boot=False)
        assert o.malloc(seg) == 0                  # segment 0, class of 16 MiB blocks
        o.free(o.malloc(64 * seg))
        assert o.malloc(63 * seg) == 65 * seg
        assert o.malloc(65 * seg) == FAIL
        sv = o.export()
        assert sv.tree_ids[0] != 0xFFFF             # segment 0 is in use
        free_bit0[name] = bool(int(sv.seg_tree_words[1]) & 1)   # bottom word 0, bit 0
    assert free_bit0 == {"reference": True, "product": False}
