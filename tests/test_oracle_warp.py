"""The oracle's model of warp-wide calls (orc_replay_warp) on the CPU.

One warp's lanes that call malloc together form one team of the reference's
warp-aggregated slice claim (gallatin.cuh:865-1078).  These checks need no
GPU; tests/test_oracle_golden.py pins the model against the reference's own
build and tests/test_gpu_parity.py the CUDA allocator against both.
"""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import PRODUCT_FIXES, WARP_FREE, WARP_MALLOC, Oracle, gen_serial_trace, gen_warp_trace


def _as_single_lane_steps(ops):
    rows = np.zeros((len(ops), 33), dtype=np.uint64)
    for i, op in enumerate(ops.tolist()):
        if op >> 63:
            rows[i, 0] = (WARP_FREE << 32) | 1
            rows[i, 1] = (op & ~(1 << 63)) * 32
        else:
            rows[i, 0] = (WARP_MALLOC << 32) | 1
            rows[i, 1] = op
    return rows.reshape(-1)


def test_single_lane_steps_equal_the_serial_replay():
    ops = gen_serial_trace(11, 3000, 60, 16, 256)
    a = Oracle(2 << 30, 42, fixes=0)
    b = Oracle(2 << 30, 42, fixes=0)
    out = a.replay_warp(_as_single_lane_steps(ops), smid=7).reshape(-1, 32)
    np.testing.assert_array_equal(out[:, 0], b.replay(ops, smid=7))
    assert (out[:, 1:] == FAIL).all()
    assert a.export().diff(b.export()) == []


def _sizes_of(size):
    return 1 << max(4, (size - 1).bit_length())


@pytest.mark.parametrize("seed,weights", [(5, (6, 4, 3, 2, 1, 1, 1, 1, 2)),
                                          (7, (0, 0, 0, 0, 0, 0, 0, 1, 3))])
def test_team_results_are_disjoint_aligned_and_in_lane_order(seed, weights):
    steps = gen_warp_trace(seed, 1500, tree_weights=weights, big_pct=50)
    o = Oracle(2 << 30, 42, fixes=PRODUCT_FIXES)
    res = o.replay_warp(steps, smid=3).reshape(-1, 32)
    rows = steps.reshape(-1, 33)
    live = {}
    for i, row in enumerate(rows):
        kind, mask = int(row[0]) >> 32, int(row[0]) & 0xFFFFFFFF
        lanes = [l for l in range(32) if (mask >> l) & 1]
        if kind == WARP_FREE:
            for l in lanes:
                live.pop(int(row[1 + l]), None)
            continue
        got = [(l, int(res[i, l])) for l in lanes if int(res[i, l]) != FAIL]
        assert len(got) == len(lanes)                          # no failures at 2 GiB
        for l, off in got:
            n = _sizes_of(int(row[1 + l]))
            assert off % min(n, 4096) == 0
            live[i * 32 + l] = (off, n)
        # single slices: lanes that landed in the same block hold consecutive
        # slices in lane order (the team's exclusive scan)
        sizes = {_sizes_of(int(row[1 + l])) for l in lanes}
        if len(sizes) == 1 and max(sizes) <= 4096:
            n = sizes.pop()
            for (_, a), (_, b) in zip(got, got[1:]):
                if a // (4096 * n) == b // (4096 * n):
                    assert b - a == n
        iv = sorted(live.values())
        for (a, na), (b, _) in zip(iv, iv[1:]):
            assert a + na <= b


def test_mixed_classes_in_one_step_are_rejected():
    row = np.zeros(33, dtype=np.uint64)
    row[0] = (WARP_MALLOC << 32) | 0b11
    row[1], row[2] = 16, 64
    with pytest.raises(ValueError):
        Oracle(1 << 30, 1).replay_warp(row)
