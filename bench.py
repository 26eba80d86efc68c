"""Benchmark: malloc+free ops/s on the mixed 16 B–4 KiB churn, one GB300.

Workload (one step): arena 128 GiB (8,192 segments of 16 MiB), 16 rounds of
4,194,304 device threads each allocating one request (size class uniform over
32 B..4 KiB, i.e. log-uniform 16 B–4 KiB rounded up to a power of two; request
sizes non-power-of-two inside the class), a fair coin (Philox4x32-10, seed 1)
freeing each live allocation before every round but the first, a uint32
payload written at malloc and checked at free, and a final drain: 64 Mi mallocs
and 64 Mi frees per step, identical requests every step.

Arena size: a block of 4,096 slices is reclaimed only when every slice in it
is freed (the reference's design), and a slice survives k rounds of 50% coin
frees with probability 2^-k, so blocks outlive ~12 rounds and this churn's
footprint reaches ~56 GB.  In 16 GiB the reference's algorithm (the oracle)
starts failing mallocs by round 4; at 64 GiB it serves all 64 Mi without a
failure.  The arena is 128 GiB (2x that) for both arms.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is the device-resident throughput of the batched path (CTA-aggregated
persistent kernels, each step one captured CUDA graph); `e2e` is the same churn
through the public C ABI entry points (gal_malloc_batched / gal_free_batched)
with each round's request sizes copied from pinned host memory inside the
timed region.  The plain per-thread path is reported beside it, at the
reference's knobs (128 pinned slots halving to 4, 16 MiB segments) and at
the batched form's knobs.
Multi-GPU: replicas only (each rank its own allocator; no collective on the
data path); `value` sums all ranks' ops over the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "malloc+free ops/sec, mixed 16B–4KiB, 1 GB300 vs plain/ref; p50/p99 malloc cycles"
ARENA = 128 << 30
N_PER_ROUND = 4 << 20
ROUNDS = 16
SEED = 1
ALLOC_SEED = 42
WORKLOAD = ("mixed-size churn: arena 128 GiB (8192 x 16 MiB segments, Gallatin<16MiB,16,4096>), "
            "16 rounds x 4,194,304 threads, 50% coin frees before each round, drain; "
            "uint32 payload written+checked")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--threads-per-round", type=int, default=N_PER_ROUND)
    p.add_argument("--rounds", type=int, default=ROUNDS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--arena-gib", type=int, default=ARENA >> 30)
    p.add_argument("--slots", type=int, default=0,
                   help="pinned slots per size class for the batched form (0: one per SM)")
    p.add_argument("--unlocked", type=int, default=16,
                   help="batched form: classes with fewer blocks per segment gather without the lock")
    p.add_argument("--segment-mib", type=int, default=64, help="batched form: segment size")
    p.add_argument("--spares", type=int, default=1, choices=[0, 1],
                   help="batched form: a service warp keeps every pinned slot's next block prepared")
    p.add_argument("--min-size", type=int, default=16, help="batched form: smallest slice")
    p.add_argument("--max-size", type=int, default=4096, help="batched form: largest slice")
    p.add_argument("--free-mode", default="warp", choices=["cta", "warp"],
                   help="batched form: frees combined per CTA (shared-memory hash) or per warp team")
    p.add_argument("--quick", action="store_true", help="headline batched steps only (profiling)")
    p.add_argument("--configs", action="store_true",
                   help="instead of the headline: the secondary workloads (tid stamp, serial "
                        "trace, large and block-size allocations, served loop, hash tables), "
                        "one JSON line")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # start timing only once the sampler is live (its first row is out),
            # then drop that row: it was taken before the timed region
            t0 = time.time()
            while not self.rows and time.time() - t0 < 5:
                time.sleep(0.005)
            self.rows.clear()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce_over_ranks(x, world, op_name):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(x, world):
    """Slowest rank's time: the whole-job clock of independent replicas."""
    return _reduce_over_ranks(x, world, "MAX")


def sum_over_ranks(x, world):
    """Ops of all replicas together."""
    return _reduce_over_ranks(x, world, "SUM")


def measured_hbm_peak():
    """HBM copy bandwidth (GB/s) measured on this GPU model (MEASURED_PEAKS.json),
    else the fallback figure of one earlier GB300 measurement."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s, one earlier GB300 copy measurement)"


def read_profile_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` at the full workload, from the committed
    ncu summary profiles/<kernel>.md (line `traffic_bytes_per_launch: N`)."""
    path = os.path.join(ROOT, "profiles", kernel + ".md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def cpu_baseline():
    """The oracle (the reference allocator's algorithm on one host thread) on a
    bounded sample of the workload, plus glibc malloc/free on every host core."""
    import ctypes as C
    from oracle import oracle as orc
    orc.build()
    L = C.CDLL(orc.LIB_PATH)
    L.orc_churn_oracle.restype = C.c_double
    L.orc_churn_oracle.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]
    L.orc_churn_glibc.restype = C.c_double
    L.orc_churn_glibc.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p]
    ops = np.zeros(4, dtype=np.uint64)
    n, r = 1 << 20, 8
    s = L.orc_churn_oracle(ARENA, n, r, SEED, ops.ctypes.data)
    oracle_v = float(ops[0] + ops[2]) / s
    cores = os.cpu_count() or 1
    ops2 = np.zeros(4, dtype=np.uint64)
    s2 = L.orc_churn_glibc(n, r, SEED, cores, ops2.ctypes.data)
    return ({"value": oracle_v, "unit": "ops/s", "cores": 1, "kind": "port",
             "sample": f"first {r} rounds of the churn at {n} threads/round then drain "
                       f"({int(ops[0] + ops[2])} ops, {s:.2f} s), the oracle's serial model"},
            {"value": float(ops2[0] + ops2[2]) / s2, "unit": "ops/s", "cores": cores,
             "sample": f"same {r} rounds x {n} requests, glibc malloc/free, payload checked "
                       f"({int(ops2[3])} mismatches, {s2:.2f} s)"})


def run_reference(args, world, rank):
    line = {"impl": "reference", "metric": METRIC, "unit": "ops/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True}
    if rank != 0:
        return None
    try:
        from oracle import refgpu
        if not refgpu.available():
            raise FileNotFoundError("reference harness cubin absent")
        ref = refgpu.RefGPU(ARENA, ALLOC_SEED, refgpu.BOOT_RACY)
        with ClockSampler(0) as clk:
            ms, st = ref.churn(args.threads_per_round, args.rounds, SEED, args.warmup, args.steps)
        ref.close()
        ops = float(st[0] + st[3])
        secs = float(ms.sum()) / 1e3
        v = ops / secs
        line.update({
            "value": v, "ms_per_step": float(ms.mean()), "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (Philox4x32-10 seed 1)",
            "config": {"workload": WORKLOAD, "path": "reference build, plain per-thread malloc/free",
                       "threads_per_round": args.threads_per_round, "rounds": args.rounds,
                       "mallocs_failed": int(st[1]), "payload_mismatch": int(st[2]),
                       "l2": "pointer table 512 MiB > 129 MB L2"},
            "cpu_baseline": {"value": v, "unit": "ops/s", "cores": 1, "kind": "reference",
                             "sample": "whole workload, the reference's own CUDA build (compiled "
                                       "from its sources into oracle/_ref) on the GPU"},
            "e2e": {"value": v, "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "clocks": clk.summary(),
        })
    except Exception as e:  # the reference build is not present: time the oracle port instead
        base, _ = cpu_baseline()
        line.update({"value": base["value"], "ms_per_step": None, "scaling": "weak",
                     "vs_baseline": None, "dtype": "u64", "data": "synthetic (Philox4x32-10 seed 1)",
                     "config": {"workload": WORKLOAD, "path": f"oracle port on the CPU ({e})"},
                     "cpu_baseline": base,
                     "e2e": {"value": base["value"], "unit": "ops/s", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0}})
    return line


def run_tables(G):
    """512 chained hash tables (2^12-2^22 pairs, seed 3), insert / delete 50% /
    reinsert: batched and per-thread node allocation at the reference's
    default knobs, the autotuner's sweep (batched form), and both forms at the
    knobs it picks."""
    from gallatin_gb300 import tables

    def keep(d):
        return {k: d[k] for k in ("ops_per_s", "ops", "op_ms", "violations", "nodes_allocated",
                                  "deleted", "ms")}

    sizes = tables.table_sizes(512, 12, 22, seed=3)
    arena = 32 << 30
    res = {"tables": 512, "pairs": int(sizes.sum())}
    for form, batched in (("batched", True), ("plain", False)):
        g = G.Gallatin.generate_on_device(arena, 42)
        try:
            res[form + "_default_knobs"] = keep(tables.run(g, sizes, 3, batched))
        finally:
            g.close()
    t0 = time.time()
    rows = tables.autotune(sizes, arena, batched=True)
    res["autotune"] = {"points": len(rows), "seconds": time.time() - t0, "best": rows[0],
                       "worst": rows[-1]}
    best = rows[0]
    knobs = dict(bytes_per_segment=best["segment_mib"] << 20, min_size=best["min_size"],
                 max_size=best["max_size"], team_width=best["team_width"])
    for form, batched in (("batched", True), ("plain", False)):
        g = G.Gallatin.generate_on_device(arena, 42, **knobs)
        try:
            res[form + "_tuned_knobs"] = keep(tables.run(g, sizes, 3, batched))
        finally:
            g.close()
    return res


def run_configs(impl):
    """The secondary workloads, one JSON line.  Ours: the 1,048,576 x 16 B tid
    stamp on 2 GiB (the drop-in per-thread path) and the time of a 4,096-op
    serial trace replayed by one thread; large and block-size allocations on
    64 GiB; the served request loop on 32 GiB; 512 chained hash tables with
    the autotuner.  --impl reference: the same stamp through the reference
    build (the reference's hash table has no delete and does not compile with
    nvcc 13, so there is no reference run of the tables)."""
    import torch
    n, rounds = 1 << 20, 20
    out = {"metric": METRIC, "configs": True}
    if impl == "reference":
        from oracle import refgpu
        out["impl"] = "reference"
        if not refgpu.available():
            out["unavailable"] = "reference build missing (make -C oracle _ref/libref_loader.so)"
            print(json.dumps(out))
            return
        ref = refgpu.RefGPU(2 << 30, 42, refgpu.BOOT_RACY)
        ref.stamp(n, 16, 1)  # untimed round: first segment gathers
        rms, rst = ref.stamp(n, 16, rounds)
        ref.close()
        out["stamp"] = {"ops_per_s": float(rst[0] + rst[3]) / (float(rms.sum()) / 1e3),
                        "malloc_ms": float(rms[0]) / rounds, "free_ms": float(rms[1]) / rounds,
                        "stamp_errors": int(rst[2]), "failed": int(rst[1]), "rounds": rounds}
        print(json.dumps(out))
        return
    import gallatin_gb300 as G
    from gallatin_gb300 import serve
    from gallatin_gb300.workloads import large_block_workload, serial_trace
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    g.bench_stamp(n, 16, 1)  # untimed round: module load and first segment gathers
    ms, st = g.bench_stamp(n, 16, rounds)
    g.close()
    out["stamp"] = {"ops_per_s": float(st[0] + st[3]) / (float(ms.sum()) / 1e3),
                    "malloc_ms": float(ms[0]) / rounds, "free_ms": float(ms[1]) / rounds,
                    "stamp_errors": int(st[2]), "failed": int(st[1]), "rounds": rounds}
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    ops_trace = serial_trace(7, 4096)
    t0 = time.time()
    offs, _ = g.replay(ops_trace)
    out["serial_trace"] = {"ops": len(ops_trace), "s": time.time() - t0,
                           "failed": int((offs[ops_trace < (1 << 63)] == G.FAIL).sum()),
                           "error_word": g.error_word()}
    g.close()
    g = G.Gallatin.generate_on_device(64 << 30, 7)
    out["large"] = large_block_workload(g)
    g.close()
    out["serve"] = serve.serve(400, arena_bytes=32 << 30, slots=32)
    out["tables"] = run_tables(G)
    torch.cuda.synchronize()
    print(json.dumps(out))


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.configs:
        import torch
        torch.cuda.set_device(local)
        run_configs(args.impl)
        return
    if args.impl == "reference":
        line = run_reference(args, world, rank)
        if line is not None:
            print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    import gallatin_gb300 as G

    N, R = args.threads_per_round, args.rounds
    arena = args.arena_gib << 30
    # the batched form runs with its tuned knobs; the plain per-thread form with
    # the reference's defaults (128 pinned slots halving to 4)
    tuned = dict(pinned_slots_first=args.slots, pinned_slots_min=args.slots if args.slots else 0,
                 gather_unlocked_below=args.unlocked, bytes_per_segment=args.segment_mib << 20,
                 min_size=args.min_size, max_size=args.max_size, spare_blocks=args.spares)
    g = G.Gallatin.generate_on_device(arena, ALLOC_SEED, **tuned)

    # one probe step: a workload that does not fit would run the out-of-memory
    # retry paths for minutes, so stop here instead
    mode = 1 | (2 if args.free_mode == "cta" else 0)
    _, probe = g.bench_churn(N, R, SEED, batched=mode, use_graph=False, warmup=0, steps=1)
    if probe.mallocs_failed or probe.payload_mismatch or probe.error_word:
        print(json.dumps({"metric": METRIC, "error": "probe step failed", "probe": probe.as_dict()}))
        sys.exit(3)

    # headline: batched + graph
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.time()
        ms, res = g.bench_churn(N, R, SEED, batched=mode, use_graph=True,
                                warmup=args.warmup, steps=args.steps)
        wall = time.time() - t0
    torch.cuda.synchronize()
    barrier(world)
    secs = max_over_ranks(res.ms_total / 1e3, world)
    ops = sum_over_ranks(float(res.mallocs_ok + res.frees), world)
    value = ops / secs
    if args.quick:
        g.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "ops/s", "quick": True,
                              "result": res.as_dict()}))
        return

    # end to end through the public C ABI with host-resident request sizes
    sizes = torch.empty(N * R, dtype=torch.int64, pin_memory=True)
    sizes.numpy()[:] = G.churn_sizes(0, N * R, SEED).view(np.int64)
    e2e_steps = max(2, args.steps // 2)
    barrier(world)
    torch.cuda.synchronize()
    ems, eres = g.bench_churn_e2e(sizes.data_ptr(), N, R, SEED, warmup=1, steps=e2e_steps,
                                  use_graph=True)
    torch.cuda.synchronize()
    barrier(world)
    esecs = max_over_ranks(eres.ms_total / 1e3, world)
    e2e_v = sum_over_ranks(float(eres.mallocs_ok + eres.frees), world) / esecs
    del sizes

    # p50/p99 per-request latency (clock64 cycles) of one full-concurrency round
    def lat(a, batched):
        mc, fc = a.bench_latency(N, SEED + 7, batched)
        return {"malloc_p50_cycles": float(np.percentile(mc, 50)),
                "malloc_p99_cycles": float(np.percentile(mc, 99)),
                "free_p50_cycles": float(np.percentile(fc, 50)),
                "free_p99_cycles": float(np.percentile(fc, 99))}
    latency = {"requests": N, "batched": lat(g, True)}

    # roofline of the dominant kernel (malloc or free phase).  HBM: algorithmic
    # bytes per launch -- malloc: 8 B pointer store + 4 B payload store per
    # request; free: 8 B pointer load per slot scanned (rounds 1..R-1 scan
    # r*N slots, the drain R*N) + 4 B payload load + 8 B pointer clear per
    # free; allocator metadata stays in L2.  L2 atomics: one counter atomic
    # per request (the per-block malloc or free counter) against the measured
    # atomic peak.
    distinct, same = G.atomic_peak()
    per_step_mallocs = res.mallocs_ok / args.steps
    hbm_peak, peak_src = measured_hbm_peak()
    free_kern = "k_churn_free_batched" if args.free_mode == "cta" else "k_churn_free_plain"
    phases = {
        "k_churn_malloc_batched": (res.ms_malloc_kernels, res.malloc_launches, res.mallocs_ok,
                                   12.0 * res.mallocs_ok),
        free_kern: (res.ms_free_kernels, res.free_launches, res.frees,
                    8.0 * N * R * (R + 1) / 2 * args.steps + 12.0 * res.frees),
    }

    def roofline_of(kern):
        ms_k, n_launch, units, alg_bytes = phases[kern]
        avg_launch_s = ms_k / 1e3 / n_launch
        achieved = (units / n_launch) / avg_launch_s
        hbm_achieved = (alg_bytes / n_launch) / avg_launch_s
        traffic = read_profile_traffic(kern)
        return {"bound": "hbm", "kernel": kern, "achieved": hbm_achieved / 1e9,
                "peak": hbm_peak, "unit": "GB/s", "frac": hbm_achieved / 1e9 / hbm_peak,
                "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes / n_launch,
                "launch_ms": avg_launch_s * 1e3,
                # the DRAM bytes ncu counted per launch over this run's launch time:
                # what the memory system moved (scattered 4 B payload accesses
                # move whole sectors)
                "dram_traffic_gbs": traffic / avg_launch_s / 1e9 if traffic else None,
                "dram_traffic_frac": traffic / avg_launch_s / 1e9 / hbm_peak if traffic else None,
                "peak_source": peak_src,
                "l2_atomic": {"achieved": achieved / 1e9, "peak": distinct / 1e9,
                              "unit": "Gatomic/s", "frac": achieved / distinct,
                              "atomics_per_unit": 1,
                              "peak_source": "measured in this run: atomicAdd.u32 with return, "
                                             "distinct addresses in a 32 MiB L2-resident buffer",
                              "same_address_peak": same / 1e9}}

    dominant = ("k_churn_malloc_batched" if res.ms_malloc_kernels >= res.ms_free_kernels
                else free_kern)
    roofline = roofline_of(dominant)
    roofline["other_phase"] = {k: v for k, v in roofline_of(
        free_kern if dominant == "k_churn_malloc_batched" else "k_churn_malloc_batched").items()
        if k not in ("peak_source",)}
    errors = g.error_word()
    g.close()

    # plain per-thread path on the reference's default knobs, stream launches
    gp = G.Gallatin.generate_on_device(arena, ALLOC_SEED)
    plain_ms, plain = gp.bench_churn(N, R, SEED, batched=False, use_graph=False,
                                     warmup=1, steps=max(1, args.steps // 2))
    plain_v = (plain.mallocs_ok + plain.frees) / (plain.ms_total / 1e3)
    latency["plain"] = lat(gp, False)
    errors |= gp.error_word()
    gp.close()
    # the same per-thread calls on the batched form's knobs
    gt = G.Gallatin.generate_on_device(arena, ALLOC_SEED, **tuned)
    _, plain_t = gt.bench_churn(N, R, SEED, batched=False, use_graph=True,
                                warmup=1, steps=max(1, args.steps // 2))
    plain_tuned_v = (plain_t.mallocs_ok + plain_t.frees) / (plain_t.ms_total / 1e3)
    latency["plain_tuned_knobs"] = lat(gt, False)
    errors |= gt.error_word() | plain_t.error_word
    if plain_t.mallocs_failed or plain_t.payload_mismatch:
        errors |= 1 << 31
    gt.close()

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (Philox4x32-10 seed 1; sizes log-uniform 16 B-4 KiB rounded to pow2)",
        "config": {"workload": WORKLOAD, "path": "batched: CTA-aggregated persistent kernels, one CUDA graph per step",
                   "pinned_slots_batched": args.slots or "one per SM", "pinned_slots_plain": "128 halving to 4 (default config: 16 MiB segments, lock-free gathers below 16 blocks per segment, no spare blocks)",
                   "batched_knobs": {"gather_unlocked_below": args.unlocked, "segment_mib": args.segment_mib,
                                     "spare_blocks": args.spares,
                                     "min_size": args.min_size, "max_size": args.max_size,
                                     "free_mode": args.free_mode},
                   "arena_bytes": arena, "threads_per_round": N, "rounds": R,
                   "l2": "no flush needed: the 512 MiB pointer table and the ~56 GB live arena footprint exceed the 129 MB L2",
                   "plain_ops_per_s": plain_v, "batched_over_plain": value / plain_v / world,
                   "plain_tuned_knobs_ops_per_s": plain_tuned_v,
                   "batched_over_plain_tuned_knobs": value / plain_tuned_v / world,
                   "mallocs_per_step": per_step_mallocs, "mallocs_failed": res.mallocs_failed,
                   "payload_mismatch": res.payload_mismatch, "device_error_word": errors,
                   "wall_s_timed": wall},
        "roofline": roofline,
        "e2e": {"value": e2e_v, "unit": "ops/s", "h2d_bytes_per_step": int(eres.h2d_bytes),
                "d2h_bytes_per_step": int(eres.d2h_bytes),
                "path": "gal_malloc_batched / gal_free_batched_n C ABI with user stamp and selection "
                        "kernels; each round's sizes copied H2D from pinned host memory, counters "
                        "read back; the selection of older rounds' slots overlaps the previous "
                        "round's allocator calls on its own stream; the step captured once as a "
                        "CUDA graph (three streams)"},
        "latency": latency,
        "gpu_launches": int(res.malloc_launches + res.free_launches),
        "clocks": clk.summary(),
    }
    if world == 1 and not args.no_cpu_baseline:
        base, glibc = cpu_baseline()
        line["cpu_baseline"] = base
        line["host_malloc_baseline"] = glibc
    print(json.dumps(line))


if __name__ == "__main__":
    main()
