"""Autotuner for the batched allocator form.

Sweeps the knobs of the batched form on a reduced run of the mixed-size churn
(same request stream and free coins as bench.py, fewer threads per round) and
ranks them by malloc+free ops/s:

  bytes_per_segment  {16, 64} MiB          (the reference's template parameter)
  min_size           {16, 128} B
  max_size           {4096, 16384} B
  pinned slots       {one per SM, 128 halving to 4}   (block-buffer breadth)
  gather_unlocked_below {0, 16}            (classes that gather without a lock)
  malloc form        {per-thread teams (registers for 3 CTAs of 256 per SM),
                      one CTA claim per class, persistent CTAs with the
                      pinned blocks cached in shared memory (4 per SM)}
                                           (aggregation width of the claims;
                                            frees in warp teams from a kernel
                                            with registers for 4 CTAs per SM)
  spare blocks       {off, on}             (block-buffer depth: a prepared next
                                            block per pinned slot)
  l2_fetch_bytes     {128, 32}             (the context's L2 fetch hint, set
                                            by every point, as it outlives
                                            the allocator)

Combinations the reference rejects (bytes_per_segment < max_size * 4096,
gallatin.cuh:300) are skipped, so 4 MiB segments drop out for max 4096.

    python -m gallatin_gb300.autotune [--threads-per-round N] [--rounds R] [--out file.json]
"""
import argparse
import itertools
import json
import sys
import time

ARENA = 128 << 30


def grid():
    for seg, mn, mx, slots, unlocked, form, spares, l2 in itertools.product(
            (16, 64), (16, 128), (4096, 16384), (0, 128), (0, 16), ("plain", "cta", "cached"), (0, 1),
            (128, 32)):
        if (seg << 20) < mx * 4096:
            continue
        yield dict(segment_mib=seg, min_size=mn, max_size=mx, slots=slots, unlocked=unlocked,
                   form=form, spares=spares, l2_fetch_bytes=l2)


# gal_bench_churn modes of the malloc forms (frees: warp teams, classes staged)
FORM_MODES = {"plain": 256 | 512, "cta": 1 | 512, "cached": 4 | 128 | 512}


def run_one(G, knobs, n, rounds, steps, seed=1):
    cfg = dict(bytes_per_segment=knobs["segment_mib"] << 20, min_size=knobs["min_size"],
               max_size=knobs["max_size"], pinned_slots_first=knobs["slots"],
               pinned_slots_min=knobs["slots"] if knobs["slots"] else 0,
               gather_unlocked_below=knobs["unlocked"], spare_blocks=knobs.get("spares", 0),
               l2_fetch_bytes=knobs.get("l2_fetch_bytes", 0))
    if knobs["slots"] == 128:
        cfg["pinned_slots_min"] = 4
    g = G.Gallatin.generate_on_device(ARENA, 42, **cfg)
    try:
        mode = FORM_MODES[knobs["form"]]
        _, r = g.bench_churn(n, rounds, seed, batched=mode, use_graph=True, warmup=1, steps=steps)
        ok = r.mallocs_failed == 0 and r.payload_mismatch == 0 and r.error_word == 0
        return {"knobs": knobs, "ops_per_s": (r.mallocs_ok + r.frees) / (r.ms_total / 1e3),
                "ms_per_step": r.ms_total / steps, "ok": ok}
    finally:
        g.close()


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--threads-per-round", type=int, default=1 << 20)
    p.add_argument("--rounds", type=int, default=16)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    import gallatin_gb300 as G
    results = []
    t0 = time.time()
    for knobs in grid():
        res = run_one(G, knobs, a.threads_per_round, a.rounds, a.steps)
        results.append(res)
        print(json.dumps(res), flush=True)
    good = sorted((r for r in results if r["ok"]), key=lambda r: -r["ops_per_s"])
    summary = {"best": good[0] if good else None, "ranked": good,
               "rejected": [r for r in results if not r["ok"]],
               "workload": f"churn {a.threads_per_round} threads/round x {a.rounds} rounds",
               "seconds": time.time() - t0}
    if a.out:
        with open(a.out, "w") as f:
            json.dump(summary, f, indent=1)
    print("BEST", json.dumps(summary["best"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
