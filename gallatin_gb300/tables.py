"""Batched uneven instances: chained hash tables served by the allocator.

512 independent tables in one launch per phase, table sizes log-uniform over
2^12-2^22 uint64 key/value pairs (seed 3), buckets of 128 B slab nodes from
the allocator; insert all, delete a random 50%, reinsert (the device side is
gallatin_gb300/csrc/gal_tables.cu, which also checks every key after the
delete and after the reinsert, and each table's live count).

The autotuner sweeps the allocator's knobs on this workload: segment size
{4, 16, 64} MiB, min size {16, 128} B, max size {4096, 16384} B and the
aggregation width of per-thread claims and frees {8, 16, 32} lanes.
Combinations the reference rejects (bytes_per_segment < max_size * 4096,
gallatin.cuh:300) are skipped, so 4 MiB segments drop out and 16,384 B slices
need 64 MiB segments: 18 legal points.

    python -m gallatin_gb300.tables [--tables 512] [--lo 12] [--hi 22] [--autotune]
"""
import argparse
import itertools
import json
import time

import numpy as np

M64 = (1 << 64) - 1


def table_sizes(n_tables=512, lo_bits=12, hi_bits=22, seed=3):
    """Pairs per table, log-uniform over [2^lo, 2^hi] (numpy PCG64 from seed)."""
    rng = np.random.default_rng(seed)
    return np.floor(2.0 ** rng.uniform(lo_bits, hi_bits, n_tables)).astype(np.uint64)


def offsets_of(sizes):
    return np.concatenate([[0], np.cumsum(sizes, dtype=np.uint64)]).astype(np.uint64)


def _mix64(z):
    """splitmix64's finaliser on uint64 numpy arrays (gal_tables.cu mix64)."""
    z = z.astype(np.uint64)
    z ^= z >> np.uint64(30)
    z *= np.uint64(0xBF58476D1CE4E5B9)
    z ^= z >> np.uint64(27)
    z *= np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    return z


def table_keys(t, n, seed=3):
    """Keys of table t (gal_tables.cu table_key)."""
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = ((np.uint64(t) << np.uint64(32)) | i) + np.uint64((seed * 0x9E3779B97F4A7C15) & M64)
        return _mix64(x)


def table_values(keys):
    with np.errstate(over="ignore"):
        return _mix64(keys ^ np.uint64(0x5851F42D4C957F2D))


def table_coins(keys):
    with np.errstate(over="ignore"):
        return (_mix64(keys + np.uint64(0x2545F4914F6CDD1D)) & np.uint64(1)).astype(bool)


def run(g, sizes, seed=3, batched=True, dump_table=None):
    """One pass of the workload on allocator g; dict of results (ops/s counts
    inserts + deletes + reinserts over their three phases)."""
    off = offsets_of(sizes)
    cap = int(sizes[dump_table]) + 8 if dump_table is not None else 0
    r, keys, vals = g.bench_tables(off, seed, batched, dump_table, cap)
    d = r.as_dict()
    ms = d["ms"]
    n = int(off[-1])
    n_del = int(d["deleted"])
    ops = n + 2 * n_del
    d["ops"] = ops
    d["op_ms"] = ms[0] + ms[1] + ms[3]
    d["ops_per_s"] = ops / (d["op_ms"] / 1e3) if d["op_ms"] > 0 else 0.0
    d["violations"] = int(d["missing"] + d["unexpected"] + d["wrong_value"] + d["count_mismatch"]
                          + d["lock_timeouts"] + d["malloc_failed"] + d["setup_failed"]
                          + (d["error_word"] != 0))
    if dump_table is not None:
        d["dump"] = (keys, vals)
    return d


def grid():
    for seg, mn, mx, width in itertools.product((4, 16, 64), (16, 128), (4096, 16384), (8, 16, 32)):
        if (seg << 20) < mx * 4096:
            continue
        yield dict(segment_mib=seg, min_size=mn, max_size=mx, team_width=width)


def autotune(sizes, arena_bytes=32 << 30, seed=3, batched=True, repeats=1, log=None):
    """Rank the legal knob settings by ops/s on this workload; each point on a
    fresh allocator."""
    import gallatin_gb300 as G
    rows = []
    for knobs in grid():
        best = None
        for _ in range(repeats):
            g = G.Gallatin.generate_on_device(arena_bytes, 42, bytes_per_segment=knobs["segment_mib"] << 20,
                                              min_size=knobs["min_size"], max_size=knobs["max_size"],
                                              team_width=knobs["team_width"])
            try:
                d = run(g, sizes, seed, batched)
            finally:
                g.close()
            if best is None or d["ops_per_s"] > best["ops_per_s"]:
                best = d
        row = dict(knobs, ops_per_s=best["ops_per_s"], violations=best["violations"],
                   nodes=best["nodes_allocated"])
        rows.append(row)
        if log:
            log(row)
    rows.sort(key=lambda r: (r["violations"] == 0, r["ops_per_s"]), reverse=True)
    return rows


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--tables", type=int, default=512)
    p.add_argument("--lo", type=int, default=12)
    p.add_argument("--hi", type=int, default=22)
    p.add_argument("--arena-gib", type=int, default=32)
    p.add_argument("--autotune", action="store_true")
    p.add_argument("--plain", action="store_true", help="per-thread node allocation")
    a = p.parse_args()
    import torch
    torch.cuda.set_device(0)
    import gallatin_gb300 as G
    sizes = table_sizes(a.tables, a.lo, a.hi)
    if a.autotune:
        t0 = time.time()
        rows = autotune(sizes, a.arena_gib << 30, batched=not a.plain,
                        log=lambda r: print(json.dumps(r), flush=True))
        print(json.dumps({"best": rows[0], "seconds": time.time() - t0}))
        return
    g = G.Gallatin.generate_on_device(a.arena_gib << 30, 42)
    try:
        d = run(g, sizes, batched=not a.plain)
    finally:
        g.close()
    print(json.dumps(d))


if __name__ == "__main__":
    main()
