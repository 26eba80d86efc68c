"""Benchmark: malloc+free ops/s on the mixed 16 B–4 KiB churn, one GB300.

Workload (one step): an arena of 128 GiB cut into 2,048 segments of 64 MiB
(Gallatin<64 MiB, 16, 4096>), 16 rounds of 4,194,304 device threads each
allocating one request (size class uniform over 32 B..4 KiB, i.e. log-uniform
16 B–4 KiB rounded up to a power of two; request sizes non-power-of-two
inside the class), a fair coin (Philox4x32-10, seed 1) freeing each live
allocation before every round but the first, a uint32 payload written at
malloc and checked at free, and a final drain: 64 Mi mallocs and 64 Mi frees
per step, identical requests every step.  Both arms run exactly this
workload and geometry (`config`); the reference arm also reports its own
default geometry (16 MiB segments).

Arena size: a block of 4,096 slices is reclaimed only when every slice in it
is freed (the reference's design), and a slice survives k rounds of 50% coin
frees with probability 2^-k, so blocks outlive ~12 rounds and this churn's
footprint reaches ~56 GB.  In 16 GiB the reference's algorithm (the oracle)
starts failing mallocs by round 4; at 64 GiB it serves all 64 Mi without a
failure.  The arena is 128 GiB (2x that) for both arms.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is the device-resident throughput of the fastest form measured (each
step one captured CUDA graph; by default malloc one thread per request in a
kernel compiled for 3 CTAs of 256 threads per SM, warp teams claiming with one
atomic each, and a persistent free phase looking segment classes up in a copy
staged in shared memory); `e2e` is the same churn through the
public C ABI entry points (gal_malloc_batched / gal_free_batched_n) with each
round's request sizes copied from pinned host memory inside the timed region.
Beside it: every malloc form at the same knobs, on the full churn and on the
allocator-only churn (no payload), the per-thread path at the reference's
default knobs, the resident server, per-request latency, and the secondary
workloads (1 Mi x 16 B stamp, large and block-size allocations, served loop)
with the reference build's figures where it has the path.
Multi-GPU: replicas only (each rank its own allocator; no collective on the
data path); `value` sums all ranks' ops over the slowest rank's time.
"""
import argparse
import faulthandler
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
SEGMENT = 64 << 20
N_PER_ROUND = 4 << 20
ROUNDS = 16
SEED = 1
ALLOC_SEED = 42
WORKLOAD = ("mixed-size churn: arena 128 GiB as 2,048 segments of 64 MiB (Gallatin<64MiB,16,4096>), "
            "16 rounds x 4,194,304 threads, sizes log-uniform 16 B-4 KiB, 50% coin frees before each "
            "round, drain; uint32 payload written+checked")
# the knobs of this library's throughput settings (gal_config); the reference has none of them
TUNED = dict(pinned_slots_first=0, pinned_slots_min=0, gather_unlocked_below=16,
             bytes_per_segment=SEGMENT, spare_blocks=1, block_layout=1, l2_fetch_bytes=32, gather_ahead=1)
# gal_bench_churn modes: bit 0 CTA claim, bit 2 cached pinned blocks, bit 3 allocator-only,
# bits 7 / 8 the plain or cached malloc kernel compiled for 4 / 3 CTAs of 256 threads per SM
FORMS = {"plain": 0, "cta": 1, "cached": 4}
SERVER_STREAMS = [          # (requests, lo, hi, log-uniform, kept for this many later requests)
    (6_000_000, 16, 128, 0, 1),
    (4_000_000, 16, 4096, 1, 2),
    (1_000_000, 1024, 32768, 1, 4),
]


def workload_config(n, r, arena):
    """The workload both arms run (identical dicts)."""
    return {"workload": WORKLOAD, "arena_bytes": arena, "segment_bytes": SEGMENT, "min_size": 16,
            "max_size": 4096, "threads_per_round": n, "rounds": r, "seed": SEED,
            "l2": "no flush needed: the 512 MiB pointer table and the ~56 GB live arena footprint exceed "
                  "the 129 MB L2"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)  # ~1 s timed: ~20 clock samples
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--threads-per-round", type=int, default=N_PER_ROUND)
    p.add_argument("--rounds", type=int, default=ROUNDS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--arena-gib", type=int, default=ARENA >> 30)
    p.add_argument("--malloc-form", default="plain", choices=["cached", "cta", "plain"],
                   help="headline malloc: persistent CTAs with cached pinned blocks, one CTA claim per "
                        "class, or one thread per request")
    p.add_argument("--ctas-per-sm", type=int, default=3, choices=[0, 3, 4],
                   help="plain and cached forms: CTAs of 256 threads per SM the malloc kernel's "
                        "registers must allow (0: the kernel's own count -- no bound for plain, 2 "
                        "for cached)")
    p.add_argument("--l2-fetch-bytes", type=int, default=32, choices=[0, 32, 64, 128],
                   help="gal_config.l2_fetch_bytes of the tuned allocators (0: leave the context's "
                        "setting)")
    p.add_argument("--gather-ahead", type=int, default=1, choices=[0, 1],
                   help="gal_config.gather_ahead of the tuned allocators")
    p.add_argument("--free-ctas-per-sm", type=int, default=4, choices=[0, 4],
                   help="free kernel: CTAs of 256 threads per SM its registers must allow (0: no bound)")
    p.add_argument("--slots", type=int, default=0,
                   help="pinned slots per class (0: one per SM); small profiling cases use fewer")
    p.add_argument("--block-layout", default="record", choices=["record", "dense"],
                   help="block counters: one 32-byte record per block, or dense arrays")
    p.add_argument("--quick", action="store_true", help="headline steps only (profiling)")
    p.add_argument("--quick-e2e", action="store_true",
                   help="headline steps, then the end-to-end C-ABI steps only (profiling)")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the secondary workloads and the reference figures beside them")
    p.add_argument("--configs", action="store_true",
                   help="only the secondary workloads (tid stamp, serial trace, large and block-size "
                        "allocations, served loop, hash tables), one JSON line")
    p.add_argument("--only", default="", help="with --configs: comma-separated subset")
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


def set_l2_fetch_bytes(nbytes):
    """Hint the largest L2 fetch for this process's context
    (cudaLimitMaxL2FetchGranularity); the setting ends with the process."""
    import ctypes as C
    cudart = C.CDLL(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"))
    rc = cudart.cudaDeviceSetLimit(C.c_int(5), C.c_size_t(nbytes))
    if rc != 0:
        raise RuntimeError(f"cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, {nbytes}) returned {rc}")


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


def cpu_baseline(n=N_PER_ROUND, r=ROUNDS):
    """The oracle (the reference allocator's algorithm, Gallatin<64 MiB, 16,
    4096>, on one host thread) on the whole workload, plus glibc malloc/free on
    every host core on the same requests."""
    import ctypes as C
    from oracle import oracle as orc
    orc.build()
    L = C.CDLL(orc.LIB_PATH)
    L.orc_churn_oracle.restype = C.c_double
    L.orc_churn_oracle.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]
    L.orc_churn_glibc.restype = C.c_double
    L.orc_churn_glibc.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p]
    ops = np.zeros(4, dtype=np.uint64)
    s = L.orc_churn_oracle(ARENA, SEGMENT, n, r, SEED, ops.ctypes.data)
    oracle_v = float(ops[0] + ops[2]) / s
    cores = os.cpu_count() or 1
    ops2 = np.zeros(4, dtype=np.uint64)
    s2 = L.orc_churn_glibc(n, r, SEED, cores, ops2.ctypes.data)
    return ({"value": oracle_v, "unit": "ops/s", "cores": 1, "kind": "port",
             "sample": f"the whole step ({r} rounds x {n} threads then drain, {int(ops[0] + ops[2])} ops, "
                       f"{s:.2f} s) served by the oracle's serial model of the reference at 64 MiB segments"},
            {"value": float(ops2[0] + ops2[2]) / s2, "unit": "ops/s", "cores": cores,
             "sample": f"the same {r} rounds x {n} requests, glibc malloc/free, payload checked "
                       f"({int(ops2[3])} mismatches, {s2:.2f} s)"})


# ---------------------------------------------------------------- reference arm
def run_reference(args, world, rank):
    line = {"impl": "reference", "metric": METRIC, "unit": "ops/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True}
    if rank != 0:
        return None
    n, r = args.threads_per_round, args.rounds
    cfg = workload_config(n, r, args.arena_gib << 30)
    try:
        from oracle import refgpu
        if not refgpu.available(64) or not refgpu.available(16):
            raise FileNotFoundError("reference harness cubins absent")

        def churn(seg_mib, steps):
            ref = refgpu.RefGPU(args.arena_gib << 30, ALLOC_SEED, refgpu.BOOT_RACY, segment_mib=seg_mib)
            try:
                return ref.churn(n, r, SEED, args.warmup, steps)
            finally:
                ref.close()

        with ClockSampler(0) as clk:
            ms, st = churn(64, args.steps)
        ops = float(st[0] + st[3])
        v = ops / (float(ms.sum()) / 1e3)
        ms16, st16 = churn(16, max(3, args.steps // 4))
        v16 = float(st16[0] + st16[3]) / (float(ms16.sum()) / 1e3)
        # the same 64 MiB churn once more with the context hint this library's
        # tuned settings give (gal_config.l2_fetch_bytes = 32); last, as the
        # hint stays for the rest of the process
        set_l2_fetch_bytes(32)
        msh, sth = churn(64, max(3, args.steps // 4))
        vh = float(sth[0] + sth[3]) / (float(msh.sum()) / 1e3)
        line.update({
            "value": v, "ms_per_step": float(ms.mean()), "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (Philox4x32-10 seed 1; sizes log-uniform 16 B-4 KiB rounded to pow2)",
            "config": cfg,
            "path": "the reference's own device code (compiled from its sources into oracle/_ref) as "
                    "Gallatin<64MiB,16,4096>, plain per-thread malloc/free",
            "mallocs_failed": int(st[1]), "payload_mismatch": int(st[2]),
            "reference_default_geometry": {
                "segment_bytes": 16 << 20, "ops_per_s": v16, "ms_per_step": float(ms16.mean()),
                "mallocs_failed": int(st16[1]), "payload_mismatch": int(st16[2]),
                "note": "the reference's global type Gallatin<16MiB,16,4096> on the same churn"},
            "reference_l2_fetch_32": {
                "segment_bytes": 64 << 20, "ops_per_s": vh, "ms_per_step": float(msh.mean()),
                "mallocs_failed": int(sth[1]), "payload_mismatch": int(sth[2]),
                "note": "the same 64 MiB churn after cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, "
                        "32), the context hint of this library's tuned settings; `value` runs without it"},
            "cpu_baseline": {"value": v, "unit": "ops/s", "cores": 1, "kind": "reference",
                             "sample": "the whole workload, the reference's own CUDA build on the GPU (it has "
                                       "no CPU implementation of this path)"},
            "e2e": {"value": v, "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "clocks": clk.summary(),
        })
    except Exception as e:  # the reference build is not present: time the oracle port instead
        base, _ = cpu_baseline()
        line.update({"value": base["value"], "ms_per_step": None, "scaling": "weak",
                     "vs_baseline": None, "dtype": "u64", "data": "synthetic (Philox4x32-10 seed 1)",
                     "config": cfg, "path": f"oracle port on the CPU ({e})",
                     "cpu_baseline": base,
                     "e2e": {"value": base["value"], "unit": "ops/s", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0}})
    return line


# The reference build is not run on the large/block workload: when a run of
# segments cannot be found, its search ends by setting bits of the segment
# tree's first word that no try had cleared (veb.cuh:447), marking segments in
# use as free; the next claim of such a segment hits one of its trap
# instructions (gallatin.cuh:1488), and a trap ends the GPU context.  This
# workload refuses run requests at its fill margin, so it would reach that.
REFERENCE_LARGE_UNAVAILABLE = ("unavailable: the reference's failed segment-run search marks in-use "
                               "segments free (veb.cuh:447) and its next claim traps (gallatin.cuh:1488)")


def reference_configs(only):
    """The reference build on the secondary workloads it has a path for: the
    1 Mi x 16 B tid stamp (its global_test flow) and the large and block-size
    allocations.  Runs in its own process (driver API)."""
    from oracle import refgpu
    out = {"impl": "reference"}
    if not refgpu.available():
        out["unavailable"] = "reference build missing (make -C oracle refcubins)"
        return out
    if "stamp" in only:
        ref = refgpu.RefGPU(2 << 30, 42, refgpu.BOOT_RACY)
        ref.stamp(1 << 20, 16, 1)  # untimed round: first segment gathers
        rms, rst = ref.stamp(1 << 20, 16, 20)
        ref.close()
        out["stamp"] = {"ops_per_s": float(rst[0] + rst[3]) / (float(rms.sum()) / 1e3),
                        "malloc_ms": float(rms[0]) / 20, "free_ms": float(rms[1]) / 20,
                        "stamp_errors": int(rst[2]), "failed": int(rst[1]), "rounds": 20}
    if "large" in only:
        out["large"] = REFERENCE_LARGE_UNAVAILABLE
    return out


def reference_configs_subprocess(only):
    """reference_configs in a child process; {} when it cannot run."""
    try:
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--configs", "--impl", "reference",
                            "--only", ",".join(only)], capture_output=True, text=True, timeout=300)
        for line in reversed(r.stdout.splitlines()):
            if line.startswith("{"):
                return json.loads(line)
        return {"unavailable": (r.stderr or r.stdout)[-300:]}
    except Exception as e:  # noqa: BLE001
        return {"unavailable": str(e)[:300]}


# ---------------------------------------------------------------- secondary workloads (ours)
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


def ours_stamp(G):
    """1,048,576 threads x malloc(16) + tid stamp, check, free; 20 rounds on a
    2 GiB arena at the reference's default knobs (its global_test flow)."""
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        g.bench_stamp(1 << 20, 16, 1)  # untimed round: module load and first segment gathers
        ms, st = g.bench_stamp(1 << 20, 16, 20)
        return {"ops_per_s": float(st[0] + st[3]) / (float(ms.sum()) / 1e3),
                "malloc_ms": float(ms[0]) / 20, "free_ms": float(ms[1]) / 20,
                "stamp_errors": int(st[2]), "failed": int(st[1]), "rounds": 20,
                "error_word": g.error_word()}
    finally:
        g.close()


def ours_large(G):
    from gallatin_gb300.workloads import large_block_workload
    g = G.Gallatin.generate_on_device(64 << 30, 7)
    try:
        return large_block_workload(g)
    finally:
        g.close()


def ours_served(G):
    from gallatin_gb300 import serve
    return serve.serve(400, arena_bytes=32 << 30, slots=32)


def run_configs(impl, only):
    """The secondary workloads, one JSON line."""
    import torch
    only = set(x for x in only.split(",") if x) or {"stamp", "serial", "large", "serve", "tables"}
    out = {"metric": METRIC, "configs": True}
    if impl == "reference":
        out.update(reference_configs(only))
        print(json.dumps(out))
        return
    import gallatin_gb300 as G
    from gallatin_gb300.workloads import serial_trace
    if "stamp" in only:
        out["stamp"] = ours_stamp(G)
    if "serial" in only:
        g = G.Gallatin.generate_on_device(2 << 30, 42)
        ops_trace = serial_trace(7, 4096)
        t0 = time.time()
        offs, _ = g.replay(ops_trace)
        out["serial_trace"] = {"ops": len(ops_trace), "s": time.time() - t0,
                               "failed": int((offs[ops_trace < (1 << 63)] == G.FAIL).sum()),
                               "error_word": g.error_word()}
        g.close()
    if "large" in only:
        out["large"] = ours_large(G)
    if "serve" in only:
        out["serve"] = ours_served(G)
    if "tables" in only:
        out["tables"] = run_tables(G)
    torch.cuda.synchronize()
    print(json.dumps(out))


# ---------------------------------------------------------------- our arm
_T0 = time.time()


def progress(what):
    """One line on stderr per phase, with the seconds since start."""
    print(f"[bench {time.time() - _T0:7.1f} s] {what}", file=sys.stderr, flush=True)


def churn_value(res):
    return (res.mallocs_ok + res.frees) / (res.ms_total / 1e3)


def churn_ok(res):
    return res.mallocs_failed == 0 and res.payload_mismatch == 0 and res.error_word == 0


def main():
    args = parse()
    # a phase that runs far longer than its usual seconds shows where it waits
    faulthandler.dump_traceback_later(240, repeat=True, file=sys.stderr)
    world, rank, local = dist_setup(args)
    if args.configs:
        if args.impl == "ours":
            import torch
            torch.cuda.set_device(local)
        run_configs(args.impl, args.only)
        return
    if args.impl == "reference":
        line = run_reference(args, world, rank)
        if line is not None:
            print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    import gallatin_gb300 as G
    TUNED["l2_fetch_bytes"] = args.l2_fetch_bytes
    TUNED["gather_ahead"] = args.gather_ahead

    N, R = args.threads_per_round, args.rounds
    arena = args.arena_gib << 30
    TUNED["block_layout"] = 1 if args.block_layout == "record" else 0
    TUNED["pinned_slots_first"] = TUNED["pinned_slots_min"] = args.slots
    occ_bit = {0: 0, 3: 256, 4: 128}[args.ctas_per_sm] | (512 if args.free_ctas_per_sm == 4 else 0)
    form_mode = {"cached": FORMS["cached"] | occ_bit, "cta": FORMS["cta"] | (occ_bit & 512),
                 "plain": FORMS["plain"] | occ_bit}
    head_mode = form_mode[args.malloc_form]
    occ_name = {0: "the kernel's own register count", 3: "3 CTAs", 4: "4 CTAs"}[args.ctas_per_sm]
    g = G.Gallatin.generate_on_device(arena, ALLOC_SEED, **TUNED)

    # one probe step: a workload that does not fit would run the out-of-memory
    # retry paths for minutes, so stop here instead
    _, probe = g.bench_churn(N, R, SEED, batched=head_mode, use_graph=False, warmup=0, steps=1)
    if probe.mallocs_failed or probe.payload_mismatch or probe.error_word:
        print(json.dumps({"metric": METRIC, "error": "probe step failed", "probe": probe.as_dict()}))
        sys.exit(3)

    # headline: persistent kernels, one CUDA graph per step
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.time()
        ms, res = g.bench_churn(N, R, SEED, batched=head_mode, use_graph=True,
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

    progress("headline done")
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
    errors = g.error_word() | eres.error_word
    if eres.mallocs_failed or eres.payload_mismatch:
        errors |= 1 << 31
    if args.quick_e2e:
        g.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "e2e": e2e_v, "quick": True,
                              "result": res.as_dict(), "e2e_result": eres.as_dict()}))
        return

    # roofline of the dominant kernel of the headline step.  HBM: algorithmic
    # bytes per launch -- malloc: 8 B pointer store + 4 B payload store per
    # request; free: 8 B pointer load + 4 B payload load per free, plus the
    # liveness words of the slots scanned, read and written back (1 bit per
    # slot each way; an upper bound on the writes).  L2 atomics:
    # one counter atomic per request (the per-block malloc or free counter)
    # against the atomic peak measured in this run.
    progress("e2e done")
    distinct, same = G.atomic_peak()
    hbm_peak, peak_src = measured_hbm_peak()
    malloc_kern = {"cached": "k_churn_malloc_cached", "cta": "k_churn_malloc_batched",
                   "plain": "k_churn_malloc_plain"}[args.malloc_form]
    free_kern = "k_churn_free_plain"
    scanned = N * R * (R + 1) / 2 * args.steps
    phases = {
        malloc_kern: (res.ms_malloc_kernels, res.malloc_launches, res.mallocs_ok, 12.0 * res.mallocs_ok),
        free_kern: (res.ms_free_kernels, res.free_launches, res.frees, scanned / 4 + 12.0 * res.frees),
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

    dominant = malloc_kern if res.ms_malloc_kernels >= res.ms_free_kernels else free_kern
    roofline = roofline_of(dominant)
    roofline["other_phase"] = {k: v for k, v in roofline_of(
        free_kern if dominant == malloc_kern else malloc_kern).items() if k not in ("peak_source",)}

    # p50/p99 per-request latency (clock64 cycles) of one full-concurrency round
    def lat(a, batched):
        mc, fc = a.bench_latency(N, SEED + 7, batched)
        return {"malloc_p50_cycles": float(np.percentile(mc, 50)),
                "malloc_p99_cycles": float(np.percentile(mc, 99)),
                "free_p50_cycles": float(np.percentile(fc, 50)),
                "free_p99_cycles": float(np.percentile(fc, 99))}
    latency = {"requests": N}
    for key, b in (("cached", 2), ("cta_claim", 1), ("plain_tuned_knobs", 0)):
        latency[key] = lat(g, b)
        progress(f"latency {key} done")
    g.close()

    # every malloc form at the same knobs, full churn and allocator-only churn
    steps_f = max(3, args.steps // 3)
    forms = {}
    for name, mode in (("plain", form_mode["plain"]), ("cta", form_mode["cta"]), ("cached", form_mode["cached"])):
        entry = {}
        for bare, key in ((0, "full"), (8, "allocator_only")):
            gf = G.Gallatin.generate_on_device(arena, ALLOC_SEED, **TUNED)
            try:
                _, rf = gf.bench_churn(N, R, SEED, batched=mode | bare, use_graph=True, warmup=1, steps=steps_f)
                errors |= rf.error_word | (0 if churn_ok(rf) else 1 << 31)
            finally:
                gf.close()
            progress(f"form {name} {key} done")
            v = churn_value(rf)
            step_ms = rf.ms_total / steps_f
            mall = rf.mallocs_ok / steps_f
            e = {"ops_per_s": v, "ms_per_step": step_ms, "malloc_kernels_ms": rf.ms_malloc_kernels / steps_f,
                 "free_kernels_ms": rf.ms_free_kernels / steps_f}
            # one claim atomic per malloc and one free-counter atomic per free,
            # over each phase's kernel time, against the in-run atomic peak
            e["malloc_l2_atomic_frac"] = mall / (rf.ms_malloc_kernels / steps_f / 1e3) / distinct
            e["free_l2_atomic_frac"] = (rf.frees / steps_f) / (rf.ms_free_kernels / steps_f / 1e3) / distinct
            entry[key] = e
        forms[name] = entry
    forms["note"] = ("same knobs for every form: one pinned slot per SM, 64 MiB segments, lock-free gathers "
                     "below 16 blocks per segment, spare blocks, one 32-byte record per block; "
                     "allocator_only = the same requests, frees and pointer stores without the payload "
                     "word; l2_atomic_frac = one counter atomic per request over the phase's kernel time "
                     "against the in-run atomicAdd peak")

    # the per-thread path at the reference's default knobs (128 pinned slots
    # halving to 4, 16 MiB segments, no spare blocks)
    progress("forms done")
    gp = G.Gallatin.generate_on_device(arena, ALLOC_SEED)
    _, plain = gp.bench_churn(N, R, SEED, batched=False, use_graph=False, warmup=1, steps=max(1, args.steps // 3))
    plain_v = churn_value(plain)
    latency["plain_default_knobs"] = lat(gp, 0)
    errors |= gp.error_word()
    gp.close()

    # the resident server against the same producers calling malloc directly
    progress("plain default knobs done")
    server = {}
    if world == 1:
        for key, direct in (("server", False), ("direct", True)):
            gs = G.Gallatin.generate_on_device(64 << 30, ALLOC_SEED, **TUNED)
            try:
                sms, sr = gs.bench_server(SERVER_STREAMS, server_pct=20, direct=direct, use_graph=True,
                                          warmup=1, steps=3)
            finally:
                gs.close()
            server[key] = {"ops_per_s": (sr.mallocs_ok + sr.frees) / (sr.ms_total / 1e3) if sr.ms_total else None,
                           "ms_per_step": sr.ms_total / 3, "violations": int(sr.stamp_mismatch + sr.misaligned + sr.not_zeroed),
                           "failed": int(sr.mallocs_failed), "status": int(sr.status),
                           "error_word": int(sr.error_word),
                           "grid": int(sr.grid), "server_ctas": int(sr.server_ctas), "graph": bool(sr.graph)}
            progress(f"server {key} done")
        server["streams"] = [list(s) for s in SERVER_STREAMS]
        server["server_pct"] = 20

    # hot-word layout: L2 atomics/s on 8-byte counters, each hit by warps of
    # its own, packed 1, 2 or 4 to a 32-byte sector (304 counters: two per SM,
    # as the pinned blocks of two classes; 1,216: eight per SM)
    hot_words = {}
    if world == 1:
        for hot in (304, 1216):
            hot_words[str(hot)] = {str(k): G.sector_probe(hot, k) / 1e9 for k in (1, 2, 4)}
        hot_words["unit"] = "Gatomic/s by counters per 32-byte sector"
        progress("hot-word probe done")

    # secondary workloads, ours and the reference build's
    configs = {}
    if world == 1 and not args.no_extras:
        configs["1_stamp"] = {"ours": ours_stamp(G)}
        progress("stamp done")
        configs["3_large"] = {"ours": ours_large(G)}
        progress("large done")
        served = ours_served(G)
        progress("served done")
        configs["5_served"] = {"ours": {k: served[k] for k in served if k != "checksums"}}
        ref = reference_configs_subprocess(["stamp"])
        progress("reference stamp done")
        configs["1_stamp"]["reference"] = ref.get("stamp", ref.get("unavailable"))
        configs["3_large"]["reference"] = REFERENCE_LARGE_UNAVAILABLE
        configs["5_served"]["reference"] = ("n/a: the reference's queue (data_structs/queue.cuh) does not "
                                            "compile with nvcc 13")

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "ops/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (Philox4x32-10 seed 1; sizes log-uniform 16 B-4 KiB rounded to pow2)",
        "config": workload_config(N, R, arena),
        "path": {"cached": "persistent malloc CTAs (256 threads, registers for %s per SM) that keep their SM's "
                           "pinned blocks in shared memory, one atomicAdd per warp team" % occ_name,
                 "cta": "persistent malloc CTAs of 512 threads, one claim per class and CTA",
                 "plain": "malloc one thread per request (256-thread CTAs, registers for %s per SM), warp "
                          "teams with one atomicAdd per team" % occ_name}[args.malloc_form]
                + "; persistent free phase, four frees per lane, segment classes staged in shared memory, "
                  "one free-counter atomic per warp team; one CUDA graph per step",
        "knobs": dict(TUNED, note="gal_config fields; pinned_slots_first=0 means one pinned slot per SM "
                                  "in every class; l2_fetch_bytes is a hint for the whole CUDA context, "
                                  "so the allocators the run builds after the headline's see it too"),
        "mallocs_per_step": res.mallocs_ok / args.steps, "mallocs_failed": int(res.mallocs_failed),
        "payload_mismatch": int(res.payload_mismatch), "device_error_word": int(errors | res.error_word),
        "wall_s_timed": wall,
        "plain_default_knobs_ops_per_s": plain_v,
        "batched_over_plain_default_knobs": value / plain_v / world,
        "batched_over_plain_same_knobs": value / forms["plain"]["full"]["ops_per_s"] / world,
        "forms_same_knobs": forms,
        "roofline": roofline,
        "e2e": {"value": e2e_v, "unit": "ops/s", "h2d_bytes_per_step": int(eres.h2d_bytes),
                "d2h_bytes_per_step": int(eres.d2h_bytes),
                "path": "gal_malloc_batched / gal_free_batched_n C ABI with user stamp and selection "
                        "kernels; each round's sizes copied H2D from pinned host memory, counters "
                        "read back; the selection of older rounds' slots overlaps the previous "
                        "round's allocator calls on its own stream; the step captured once as a "
                        "CUDA graph (three streams)"},
        "latency": latency,
        "server": server,
        "hot_word_probe": hot_words,
        "configs_secondary": configs,
        "gpu_launches": int(res.malloc_launches + res.free_launches),
        "clocks": clk.summary(),
    }
    if world == 1 and not args.no_cpu_baseline:
        base, glibc = cpu_baseline(N, R)
        progress("cpu baseline done")
        line["cpu_baseline"] = base
        line["host_malloc_baseline"] = glibc
    print(json.dumps(line))


if __name__ == "__main__":
    main()
