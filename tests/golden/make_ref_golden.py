"""Generate golden fixtures from the reference allocator's own CUDA build.

Run on a machine with a GPU, after building the reference harness where the
reference sources are (make -C oracle _ref/ref_harness.cubin):

    python tests/golden/make_ref_golden.py [outdir]

For every case it builds the reference's Gallatin<16 MiB, 16, 4096> on the
device (oracle/ref_harness.cu), records the state after boot, replays a
serial trace with one device thread and records the offsets it returned
(pointer - arena base), the SM it ran on, and the final state.  The warp
cases replay traces of warp-wide calls with one warp instead (the lanes of a
step join one team of the warp-aggregated slice claim) and go to
warp_*.npz / warp_index.json.  The files written here are the fixtures
checked by tests/test_oracle_golden.py.  Names given after the output folder
select cases; their entries are merged into the index files already there.
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refgpu  # noqa: E402
from oracle.oracle import Oracle, gen_log_trace, gen_serial_trace, gen_warp_trace  # noqa: E402

GiB = 1 << 30


def exhaust_trace():
    """On 16 segments (all taken by the boot): 20,520 mallocs of 4 KiB run the
    4 KiB class dry, 8,192 frees return two whole blocks (and their segments),
    then 4 KiB mallocs (the emptied pinned slots stay empty), whole-block and
    multi-segment requests that reuse the returned segments, and their frees."""
    ops = [4096] * 20520
    ops += [(1 << 63) | i for i in range(8192)]
    ops += [4096] * 20
    big = len(ops)
    ops += [16 << 20, 8 << 20, (16 << 20) + 1, 64 << 10]
    ops += [(1 << 63) | (big + i) for i in range(4)]
    ops += [(32 << 20), 4096, 1 << 20]
    return np.array(ops, dtype=np.uint64)


def hidden_by_return_trace():
    """On 128 segments with no pinned blocks: a run of 34 segments (94-127), a
    run of 36 (58-93, which empties bottom word 1 of the segment tree), the
    second run freed (word 1 refilled with 64-93 but not full), then 100 whole
    16 MiB blocks.  The reference lists a refilled word in the summary layer
    only when it is full (veb.cuh:1128-1154), so its single-segment searches
    reach 64 of them; with every refilled word listed, 94."""
    seg = 16 << 20
    ops = [34 * seg, 36 * seg, (1 << 63) | 1] + [seg] * 100
    return np.array(ops, dtype=np.uint64)


CASES = [
    # name, arena bytes, alloc seed, boot, trace builder
    ("cfg1_serial", 2 * GiB, 42, refgpu.BOOT_ONE_THREAD, lambda: gen_serial_trace(7, 4096, 60, 16, 256)),
    ("churn_16", 2 * GiB, 42, refgpu.BOOT_ONE_THREAD, lambda: gen_serial_trace(11, 100000, 50, 16, 1)),
    ("churn_4k", 2 * GiB, 42, refgpu.BOOT_ONE_THREAD, lambda: gen_serial_trace(13, 60000, 50, 4096, 1)),
    ("mixed_small", 2 * GiB, 42, refgpu.BOOT_ONE_THREAD, lambda: gen_serial_trace(19, 40000, 52, 16, 256)),
    ("tiers", 16 * GiB, 42, refgpu.BOOT_ONE_THREAD, lambda: gen_log_trace(17, 3000, 55, 4, 26)),
    ("exhaust_4k", 256 << 20, 42, refgpu.BOOT_ONE_THREAD, exhaust_trace),
    ("cfg1_racy_boot", 2 * GiB, 42, refgpu.BOOT_RACY, lambda: gen_serial_trace(7, 4096, 60, 16, 256)),
    ("run_return_hidden", 2 * GiB, 42, refgpu.BOOT_NONE, hidden_by_return_trace),
]

# cases whose trace reaches a reference defect that the product fixes: the
# product's offsets differ there by design
REACHES_FIX = {"run_return_hidden": "FIX_RUN_RETURN_SUMMARY"}


WARP_CASES = [
    # name, arena bytes, alloc seed, steps builder (one warp, one-thread boot)
    ("warp_mixed", 2 * GiB, 42, lambda: gen_warp_trace(5, 3000)),
    ("warp_small", 2 * GiB, 42, lambda: gen_warp_trace(6, 4000, tree_weights=(8, 4, 0, 0, 0, 0, 0, 0, 0))),
    ("warp_big", 2 * GiB, 42,
     lambda: gen_warp_trace(7, 2500, tree_weights=(0, 0, 0, 0, 0, 0, 0, 1, 3), big_pct=50)),
    ("warp_exhaust", 256 << 20, 42,
     lambda: gen_warp_trace(8, 800, malloc_pct=85, tree_weights=(0, 0, 0, 0, 0, 0, 1, 1, 4), big_pct=40)),
]


def _merge_index(path, entries):
    index = json.load(open(path)) if os.path.exists(path) else {}
    index.update(entries)
    with open(path, "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


def warp_cases(out_dir, only):
    index = {}
    for name, nbytes, seed, mk in WARP_CASES:
        if only and name not in only:
            continue
        t0 = time.time()
        steps = mk()
        rows = steps.reshape(-1, 33)
        dims = Oracle(nbytes, seed, boot=False).dims()
        ref = refgpu.RefGPU(nbytes, seed, refgpu.BOOT_ONE_THREAD)
        boot_state = ref.export(dims)
        offsets, smid = ref.replay_warp(steps)
        final_state = ref.export(dims)
        ref.close()
        boot_state.to_npz(os.path.join(out_dir, f"{name}.boot.npz"))
        final_state.to_npz(os.path.join(out_dir, f"{name}.final.npz"), ops=steps, offsets=offsets,
                           smid=np.array([smid], dtype=np.uint32))
        mall = (rows[:, 0] >> np.uint64(32)) == 0
        lanes = (rows[:, 0:1] >> np.arange(32, dtype=np.uint64)) & np.uint64(1)
        active = (lanes == 1) & mall[:, None]
        res = offsets.reshape(-1, 32)
        index[name] = {"arena_bytes": nbytes, "seed": seed, "boot": refgpu.BOOT_ONE_THREAD, "smid": smid,
                       "steps": int(len(rows)), "mallocs": int(active.sum()),
                       "failed_mallocs": int((active & (res == np.uint64((1 << 64) - 1))).sum()),
                       "seconds": round(time.time() - t0, 2)}
        print(name, index[name], flush=True)
    if index:
        _merge_index(os.path.join(out_dir, "warp_index.json"), index)


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    only = set(sys.argv[2:])
    os.makedirs(out_dir, exist_ok=True)
    index = {}
    for name, nbytes, seed, boot, mk in CASES:
        if only and name not in only:
            continue
        t0 = time.time()
        ops = mk()
        dims = Oracle(nbytes, seed, boot=False).dims()
        ref = refgpu.RefGPU(nbytes, seed, boot)
        boot_state = ref.export(dims)
        offsets, smid = ref.replay(ops)
        final_state = ref.export(dims)
        ref.close()
        boot_state.to_npz(os.path.join(out_dir, f"{name}.boot.npz"))
        final_state.to_npz(os.path.join(out_dir, f"{name}.final.npz"), ops=ops, offsets=offsets,
                           smid=np.array([smid], dtype=np.uint32))
        index[name] = {"arena_bytes": nbytes, "seed": seed, "boot": boot, "smid": smid,
                       "nops": int(len(ops)),
                       "mallocs": int((ops < (1 << 63)).sum()),
                       "failed_mallocs": int(((ops < (1 << 63)) & (offsets == (1 << 64) - 1)).sum()),
                       "seconds": round(time.time() - t0, 2)}
        if name in REACHES_FIX:
            index[name]["reaches_fix"] = REACHES_FIX[name]
        print(name, index[name], flush=True)
    if index:
        _merge_index(os.path.join(out_dir, "index.json"), index)
    warp_cases(out_dir, only)


if __name__ == "__main__":
    main()
