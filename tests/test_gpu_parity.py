"""Serial parity of the CUDA allocator (through the C ABI) on the GPU.

A trace replayed by one device thread must return the reference build's
offsets byte for byte and leave the same state, word for word:
  * against the fixtures recorded from the reference's own CUDA build
    (tests/golden/, see make_ref_golden.py), with the pinned-slot SM id set to
    the one the reference ran on;
  * against the CPU oracle (product mode) on further random traces, at the SM
    id this run landed on.
"""
import json
import os

import numpy as np
import pytest

from gallatin_gb300._abi import FAIL, GAL_POLICY_LOWEST, StateView
from oracle.oracle import (PRODUCT_FIXES, Oracle, gen_leftover_trace, gen_log_trace, gen_serial_trace,
                           gen_warp_trace)

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(GOLD, "index.json")))
_WARP = os.path.join(GOLD, "warp_index.json")
WARP_INDEX = json.load(open(_WARP)) if os.path.exists(_WARP) else {}


@pytest.fixture(scope="module")
def G():
    import gallatin_gb300
    return gallatin_gb300


def _golden(name):
    boot, _ = StateView.from_npz(os.path.join(GOLD, f"{name}.boot.npz"))
    final, z = StateView.from_npz(os.path.join(GOLD, f"{name}.final.npz"))
    return boot, final, z["ops"], z["offsets"], int(z["smid"][0])


@pytest.mark.parametrize("name", sorted(n for n in INDEX if "reaches_fix" not in INDEX[n]))
def test_serial_trace_matches_reference_build(G, name):
    meta = INDEX[name]
    boot, final, ops, offsets, smid = _golden(name)
    one_thread = meta["boot"] == 1
    g = G.Gallatin.generate_on_device(meta["arena_bytes"], meta["seed"], boot=one_thread,
                                      smid_override=smid)
    try:
        if one_thread:
            assert g.export().diff(boot) == [], "boot state differs from the reference build"
        else:
            g.load(boot)
        out, _ = g.replay(ops)
        np.testing.assert_array_equal(out, offsets)
        assert g.export().diff(final) == [], "final state differs from the reference build"
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("name", sorted(n for n in INDEX if "reaches_fix" in INDEX[n]))
def test_fixed_defect_traces_match_the_fixed_oracle(G, name):
    """Fixtures whose trace reaches a reference defect the product fixes (the
    oracle's reference mode reproduces the reference build there): from the
    same boot state, the product gives the fixed oracle's offsets and state."""
    meta = INDEX[name]
    boot, _, ops, _, smid = _golden(name)
    g = G.Gallatin.generate_on_device(meta["arena_bytes"], meta["seed"], boot=False, smid_override=smid)
    try:
        g.load(boot)
        out, _ = g.replay(ops)
        o = Oracle(meta["arena_bytes"], meta["seed"], fixes=PRODUCT_FIXES, boot=False)
        o.load(boot)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


TRACES = [
    ("serial_s101", 2 << 30, lambda: gen_serial_trace(101, 20000, 55, 16, 256)),
    ("serial_s202_16", 2 << 30, lambda: gen_serial_trace(202, 30000, 50, 16, 1)),
    ("log_4_15", 2 << 30, lambda: gen_log_trace(303, 20000, 52, 4, 15)),
    ("log_4_26", 16 << 30, lambda: gen_log_trace(404, 4000, 55, 4, 26)),
    ("log_big_small_arena", 1 << 30, lambda: gen_log_trace(505, 3000, 60, 10, 24)),
]


@pytest.mark.parametrize("name,nbytes,mk", TRACES, ids=[t[0] for t in TRACES])
def test_serial_trace_matches_oracle(G, name, nbytes, mk):
    ops = mk()
    g = G.Gallatin.generate_on_device(nbytes, 42)
    try:
        out, smid = g.replay(ops)
        o = Oracle(nbytes, 42, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


def test_lowest_policy_matches_oracle(G):
    ops = gen_serial_trace(606, 30000, 50, 4096, 1)
    g = G.Gallatin.generate_on_device(2 << 30, 9, subtree_policy=GAL_POLICY_LOWEST)
    try:
        out, smid = g.replay(ops)
        o = Oracle(2 << 30, 9, fixes=PRODUCT_FIXES, policy=GAL_POLICY_LOWEST)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
    finally:
        g.close()


@pytest.mark.parametrize("geom", [(64 << 20, 16, 4096), (64 << 20, 128, 16384), (16 << 20, 128, 4096)])
def test_other_geometries_match_oracle(G, geom):
    seg, mn, mx = geom
    ops = gen_log_trace(707, 8000, 55, 4, 20)
    g = G.Gallatin.generate_on_device(4 << 30, 3, bytes_per_segment=seg, min_size=mn, max_size=mx)
    try:
        out, smid = g.replay(ops)
        o = Oracle(4 << 30, 3, bytes_per_segment=seg, min_size=mn, max_size=mx, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
    finally:
        g.close()


@pytest.mark.parametrize("max_size", [4096, 1024])
def test_leftover_credit_completes_block(G, max_size):
    """A run that does not fit credits its leftover slices; when they are the
    last the block was owed, the block goes back to its segment (the
    reference leaks it, block.cuh:267-281)."""
    ops = gen_leftover_trace(max_size)
    g = G.Gallatin.generate_on_device(1 << 30, 5, max_size=max_size)
    try:
        out, smid = g.replay(ops)
        o = Oracle(1 << 30, 5, max_size=max_size, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        sv = g.export()
        assert sv.diff(o.export()) == []
        assert (sv.free_counters < 4096).all()
        assert g.error_word() == 0
    finally:
        g.close()


def test_state_roundtrip_export_import(G):
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        g.replay(gen_serial_trace(11, 5000, 60, 16, 256))
        sv = g.export()
        h = G.Gallatin.generate_on_device(2 << 30, 42, boot=False)
        try:
            h.load(sv)
            assert h.export().diff(sv) == []
        finally:
            h.close()
    finally:
        g.close()


def _free_everything(ops):
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
], ids=["serial", "log_big"])
def test_trim_matches_oracle_and_fresh_state(G, mk, nbytes):
    """Free everything, trim: the whole state equals the oracle's, and the
    trees, segment classes, slots and free counters equal a fresh allocator's."""
    ops = _free_everything(mk())
    g = G.Gallatin.generate_on_device(nbytes, 42)
    try:
        fresh = g.export()
        out, smid = g.replay(ops)
        g.trim()
        o = Oracle(nbytes, 42, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        o.trim()
        sv = g.export()
        assert sv.diff(o.export()) == []
        assert sv.diff(fresh, fields=["seg_tree_words", "sub_tree_words", "tree_ids", "slots",
                                      "free_counters"]) == []
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("name", sorted(WARP_INDEX))
def test_warp_trace_matches_reference_build(G, name):
    """Warp-wide calls by one warp: the lanes of a step form one team of the
    warp-aggregated claim; offsets and whole state equal the reference build's."""
    meta = WARP_INDEX[name]
    boot, final, steps, offsets, smid = _golden(name)
    g = G.Gallatin.generate_on_device(meta["arena_bytes"], meta["seed"], smid_override=smid)
    try:
        assert g.export().diff(boot) == [], "boot state differs from the reference build"
        out, _ = g.replay_warp(steps)
        np.testing.assert_array_equal(out, offsets)
        assert g.export().diff(final) == [], "final state differs from the reference build"
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("geom", [(64 << 20, 16, 4096), (64 << 20, 128, 16384), (16 << 20, 128, 4096)])
def test_warp_traces_on_other_geometries_match_oracle(G, geom):
    seg, mn, mx = geom
    trees = (mx // mn).bit_length()
    steps = gen_warp_trace(909, 1500, tree_weights=(3,) + (1,) * (trees - 2) + (3,), big_pct=40,
                           min_size=mn)
    g = G.Gallatin.generate_on_device(4 << 30, 3, bytes_per_segment=seg, min_size=mn, max_size=mx)
    try:
        out, smid = g.replay_warp(steps)
        o = Oracle(4 << 30, 3, bytes_per_segment=seg, min_size=mn, max_size=mx, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay_warp(steps, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("kind", ["serial", "warp"])
def test_one_slot_per_sm_geometry_matches_oracle(G, kind):
    """The throughput geometry (64 MiB segments, one pinned slot per SM in
    every class, lock-free gathers) without spare blocks: serial and warp-team
    traces equal the oracle with as many slots as the GPU has SMs."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = dict(bytes_per_segment=64 << 20, pinned_slots_first=0, pinned_slots_min=0,
               gather_unlocked_below=16)
    g = G.Gallatin.generate_on_device(16 << 30, 5, **cfg)
    try:
        o = Oracle(16 << 30, 5, bytes_per_segment=64 << 20, pinned_first=sms, pinned_min=sms,
                   fixes=PRODUCT_FIXES)
        assert g.export().diff(o.export()) == []       # the same boot
        if kind == "serial":
            ops = gen_log_trace(808, 20000, 55, 4, 20)
            out, smid = g.replay(ops)
            np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        else:
            steps = gen_warp_trace(818, 2500, tree_weights=(4, 2, 1, 1, 1, 1, 1, 2, 3), big_pct=40)
            out, smid = g.replay_warp(steps)
            np.testing.assert_array_equal(out, o.replay_warp(steps, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("kind", ["serial", "warp"])
def test_spare_blocks_match_oracle(G, kind):
    """spare_blocks = 1 on the per-thread path: the block that crosses slice
    4095 is replaced by the slot's prepared spare and the next spare is
    requested at once; the oracle's model of it gives the same offsets and
    state, and so does a trim afterwards (spares retired first)."""
    g = G.Gallatin.generate_on_device(2 << 30, 42, spare_blocks=1)
    try:
        o = Oracle(2 << 30, 42, fixes=PRODUCT_FIXES, spares=True)
        if kind == "serial":
            ops = gen_serial_trace(909, 30000, 58, 16, 256)
            out, smid = g.replay(ops)
            np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        else:
            steps = gen_warp_trace(919, 3000, tree_weights=(6, 3, 1, 1, 1, 1, 1, 2, 3), big_pct=40)
            out, smid = g.replay_warp(steps)
            np.testing.assert_array_equal(out, o.replay_warp(steps, smid=smid))
        assert g.export().diff(o.export()) == []
        g.trim()
        o.trim()
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


def test_run_below_the_arena_fails_and_gives_back_what_it_took(G):
    """A multi-segment request that would need segments below segment 0 (the
    reference indexes bottom-layer word -1, veb.cuh:382-410): it fails, the
    words it took are given back, and the whole state equals the oracle's."""
    from tests.test_oracle_runs import RUN_BELOW_ARENA, SEG, runs_to_ops
    ops, idx = runs_to_ops(RUN_BELOW_ARENA + [("m", 84), ("m", 64)])
    g = G.Gallatin.generate_on_device(2 << 30, 42, boot=False)
    try:
        out, smid = g.replay(ops)
        o = Oracle(2 << 30, 42, fixes=PRODUCT_FIXES, boot=False)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert int(out[idx[-2]]) == FAIL and int(out[idx[-1]]) == SEG
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


def test_a_returned_run_lists_every_word_it_refills(G):
    """Freeing a run lists every bottom word it leaves non-empty, not only the
    full ones (veb.cuh:1128-1154): after the run pair that empties word 1, the
    single-segment requests reach all 94 free segments, as in the oracle."""
    from tests.test_oracle_runs import HIDDEN_BY_RETURN, SEG, runs_to_ops
    ops, _ = runs_to_ops(HIDDEN_BY_RETURN + [("m", 1)] * 100)
    g = G.Gallatin.generate_on_device(2 << 30, 42, boot=False)
    try:
        out, smid = g.replay(ops)
        o = Oracle(2 << 30, 42, fixes=PRODUCT_FIXES, boot=False)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        singles = out[3:]
        assert int((singles != FAIL).sum()) == 94
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()


@pytest.mark.parametrize("seed", [3, 9])
def test_tier_trace_matches_the_oracle(G, seed):
    """1,500 serial requests over every tier (slices, blocks, segment runs)
    with frees in random order: offsets and whole state equal the oracle's."""
    from tests.test_oracle_fuzz import tier_trace
    nbytes = [2 << 30, 4 << 30][seed % 2]
    ops = tier_trace(seed)
    g = G.Gallatin.generate_on_device(nbytes, 42)
    try:
        out, smid = g.replay(ops)
        o = Oracle(nbytes, 42, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0
    finally:
        g.close()
