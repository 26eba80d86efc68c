"""The CPU oracle against fixtures produced by the reference's own CUDA build.

tests/golden/*.npz were written by tests/golden/make_ref_golden.py, which ran
the reference allocator (compiled from its sources) on a GB300: state after
boot, the offset every malloc of a serial trace returned, the SM the trace ran
on, and the state after the trace.  The warp_* fixtures replay traces of
warp-wide calls with one warp instead: the lanes of a step form one team of
the warp-aggregated slice claim.  The oracle in pure-reference mode
(fixes=0) must reproduce all of it bit for bit.
"""
import json
import os

import numpy as np
import pytest

from gallatin_gb300._abi import FAIL, StateView
from oracle.oracle import PRODUCT_FIXES, Oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INDEX = json.load(open(os.path.join(GOLD, "index.json")))
_WARP = os.path.join(GOLD, "warp_index.json")
WARP_INDEX = json.load(open(_WARP)) if os.path.exists(_WARP) else {}


def load_case(name):
    boot, _ = StateView.from_npz(os.path.join(GOLD, f"{name}.boot.npz"))
    final, z = StateView.from_npz(os.path.join(GOLD, f"{name}.final.npz"))
    return boot, final, z["ops"], z["offsets"], int(z["smid"][0])


@pytest.mark.parametrize("name", sorted(INDEX))
def test_oracle_matches_reference_build(name):
    meta = INDEX[name]
    boot, final, ops, offsets, smid = load_case(name)
    one_thread = meta["boot"] == 1
    o = Oracle(meta["arena_bytes"], meta["seed"], fixes=0, boot=one_thread)
    if one_thread:
        assert o.export().diff(boot) == []          # boot state equal word for word
    else:
        o.load(boot)                                 # racy boot: import its state
    out = o.replay(ops, smid=smid)
    np.testing.assert_array_equal(out, offsets)      # every offset equal
    assert o.export().diff(final) == []              # whole final state equal


@pytest.mark.parametrize("name", sorted(n for n in INDEX if "reaches_fix" not in INDEX[n]))
def test_product_fixes_do_not_change_golden_traces(name):
    """The reference defects the product fixes are not reached by these traces,
    so the product's oracle mode must give the same offsets here."""
    meta = INDEX[name]
    boot, final, ops, offsets, smid = load_case(name)
    o = Oracle(meta["arena_bytes"], meta["seed"], fixes=PRODUCT_FIXES, boot=meta["boot"] == 1)
    if meta["boot"] != 1:
        o.load(boot)
    np.testing.assert_array_equal(o.replay(ops, smid=smid), offsets)


def test_racy_boot_state_is_consistent():
    """The reference's racy <<<1,128>>> boot is nondeterministic (on the GB300
    it gave size class 0 two segments where the one-thread order gives one),
    but every pinned block it installs lies in a segment owned by its class."""
    racy, _, _, _, _ = load_case("cfg1_racy_boot")
    bps = racy.dims.blocks_per_segment
    for t in range(racy.dims.num_trees):
        slots = racy.slots_of(t)
        assert (slots >= 0).all()
        assert (racy.tree_ids[slots // bps] == t).all()
        assert len(set(slots.tolist())) == len(slots)


def test_golden_serial_trace_has_no_failures():
    _, _, ops, offsets, _ = load_case("cfg1_serial")
    m = ops < (1 << 63)
    assert m.sum() == 2456 and not (offsets[m] == FAIL).any()


@pytest.mark.parametrize("name", sorted(WARP_INDEX))
def test_oracle_warp_teams_match_reference_build(name):
    """One warp of the reference build: every lane's offset (lane-order scan
    of the team, one atomic per team, block replacement by the team's lowest
    lane with its own thread id) and the whole state after the trace."""
    meta = WARP_INDEX[name]
    boot, final, steps, offsets, smid = load_case(name)
    o = Oracle(meta["arena_bytes"], meta["seed"], fixes=0)
    assert o.export().diff(boot) == []
    out = o.replay_warp(steps, smid=smid)
    np.testing.assert_array_equal(out, offsets)
    assert o.export().diff(final) == []
    p = Oracle(meta["arena_bytes"], meta["seed"], fixes=PRODUCT_FIXES)
    np.testing.assert_array_equal(p.replay_warp(steps, smid=smid), offsets)


def test_run_return_rule_pinned_by_the_reference_build():
    """The reference build lists a segment-tree word refilled by a freed run in
    the summary layer only when the word is full (veb.cuh:1128-1154): after
    runs of 34 and 36 segments on 128 and a free of the second, its whole-block
    requests of 16 MiB reach 64 segments.  The oracle's reference mode gives
    those offsets (test above); its product mode, which lists every refilled
    word, serves 94 and agrees on everything before the requests that differ."""
    if "run_return_hidden" not in INDEX:
        pytest.skip("fixture not recorded")
    meta = INDEX["run_return_hidden"]
    boot, _, ops, offsets, smid = load_case("run_return_hidden")
    singles = ops[3:]
    assert (singles == 16 << 20).all()
    assert int((offsets[3:] != FAIL).sum()) == 64 and meta["failed_mallocs"] == 36
    o = Oracle(meta["arena_bytes"], meta["seed"], fixes=PRODUCT_FIXES, boot=False)
    o.load(boot)
    fixed = o.replay(ops, smid=smid)
    np.testing.assert_array_equal(fixed[:3], offsets[:3])
    assert int((fixed[3:] != FAIL).sum()) == 94
    live = np.concatenate([fixed[:1], fixed[3:][fixed[3:] != FAIL]])  # the second run was freed
    assert len(set(live.tolist())) == len(live)
