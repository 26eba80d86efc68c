"""Served request loop over the device allocator (continuous batching).

Jobs arrive as a Poisson process (default mean 2,000 jobs/s, seed 5).  A job is
either a device vector of uint32 grown by push_back to n elements (n
log-uniform over 1K-16M, capacity doubling through the allocator) or a queue
of 32 B nodes with n enqueue/dequeue operations (n log-uniform over 1K-4M);
each runs as a grid of up to 8 CTAs (gal_job_launch, gal_job_ctas) on a stream
slot.  The loop keeps every
slot busy: a job that has arrived is admitted as soon as a slot is free and the
arena bytes reserved by running jobs plus its own estimated footprint fit in
the budget, so jobs arriving while others run overlap with them on the device.
Allocator state stays resident on the device across all jobs.

Reported: malloc+free ops/s over the whole run; job latency (host-observed
completion - arrival) p50/p99, split into the admission wait (admission -
arrival, the host loop) and the job's device time (CUDA events around its
launch on its stream); per-request malloc/free latency p50/p99 in SM cycles
over every malloc and free of every job (clock64 around each call, counted in
a device histogram of four bins per power of two); failures.  `solo_check`
reruns jobs one at a time and compares their checksums with the mixed run.
"""
import ctypes as C
import time
from collections import deque

import numpy as np

from . import GAL_OK, Gallatin, GalError, lib

JOB_VECTOR, JOB_QUEUE = 0, 1
LAT_BINS = 160   # GAL_JOB_LAT_BINS
SEG = 16 << 20


def job_ctas(kind, n):
    """CTAs of a job (gal_job_ctas): one per 2^20 vector elements or 2^18
    queue operations, 1 to 8."""
    g = n >> 20 if kind == JOB_VECTOR else n >> 18
    return int(min(8, max(1, g)))


def lat_bin(c):
    """Histogram bin of c cycles, as gal_job_launch bins them."""
    if c < 4:
        return int(c)
    e = int(c).bit_length() - 1
    return min(4 * e + ((int(c) >> (e - 2)) & 3), LAT_BINS - 1)


def bin_value(b):
    """Cycles a latency bin stands for (the middle of its range; gal_job_launch
    puts c cycles in bin c below 4, else in 4 floor(log2 c) + the two bits
    below the leading one)."""
    if b < 4:
        return float(b)
    e, m = b // 4, b % 4
    lo = (1 << e) + m * (1 << (e - 2))
    return lo + ((1 << (e - 2)) - 1) / 2.0


def hist_percentile(counts, q):
    """q-th percentile (0-100) of a latency histogram, as its bin's value."""
    counts = np.asarray(counts, dtype=np.float64)
    total = counts.sum()
    if total == 0:
        return None
    b = int(np.searchsorted(np.cumsum(counts), q / 100.0 * total, side="left"))
    return bin_value(min(b, len(counts) - 1))


def make_jobs(num_jobs, rate=2000.0, seed=5, vector_share=0.5):
    rng = np.random.default_rng(seed)
    arrival = np.cumsum(rng.exponential(1.0 / rate, num_jobs))
    kind = np.where(rng.random(num_jobs) < vector_share, JOB_VECTOR, JOB_QUEUE)
    n_vec = 2 ** rng.uniform(10, 24, num_jobs)   # 1K .. 16M elements
    n_q = 2 ** rng.uniform(10, 22, num_jobs)     # 1K .. 4M operations
    n = np.where(kind == JOB_VECTOR, n_vec, n_q).astype(np.int64)
    return [dict(id=i, kind=int(kind[i]), n=int(n[i]), arrival=float(arrival[i])) for i in range(num_jobs)]


def footprint(kind, n):
    """Peak arena bytes a job can hold (admission estimate)."""
    if kind == JOB_VECTOR:
        g = job_ctas(kind, n)
        share = -(-n // g)                        # elements of the largest CTA share
        cap = max(1024, 1 << int(np.ceil(np.log2(max(share, 1)))))
        new, old = 4 * cap, 2 * cap              # bytes of the last two buffers of a CTA
        r = lambda b: ((b - 1) // SEG + 1) * SEG if b > SEG else 1 << int(np.ceil(np.log2(b)))
        return g * (r(new) + r(old))
    return 32 * n + SEG                           # every operation an enqueue, at most


def vector_checksum(job_id, n):
    """Host value of a vector job's checksum (sum of its pushed values)."""
    j = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = np.uint64(job_id) * np.uint64(0x9E3779B97F4A7C15) + j * np.uint64(0xBF58476D1CE4E5B9) \
            + np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
        x *= np.uint64(0xD6E8FEB86659FD93)
    return int((x >> np.uint64(32)).sum(dtype=np.uint64))


def schedule(jobs, slots, budget, launch, clock, realtime=True, limit_s=None):
    """The admission loop.  jobs: dicts with kind, n, arrival and row.  A job is
    admitted in arrival order once it has arrived (realtime) or at once, as
    soon as a slot is free and the estimated footprints of the running jobs
    plus its own fit in `budget`; a job that does not fit even alone runs
    alone.  launch(job, slot) starts it and returns an object whose query()
    says whether it has finished; clock() gives seconds since the start.
    Returns the admission and completion times per row and the most jobs that
    ran at once.  With limit_s, a loop still waiting after that many seconds
    raises TimeoutError instead of polling on."""
    nj = len(jobs)
    pending = deque(sorted(jobs, key=lambda j: j["arrival"]))
    free_slots = list(range(slots))
    running = {}
    reserved = 0
    admit_t, done_t = np.zeros(nj), np.zeros(nj)
    max_running = 0
    while pending or running:
        now = clock()
        if limit_s is not None and now > limit_s:
            raise TimeoutError(f"served loop: {len(pending)} jobs pending and {len(running)} running "
                               f"after {now:.0f} s")
        for slot, (job, ev) in list(running.items()):
            if ev.query():
                done_t[job["row"]] = clock()
                reserved -= job["est"]
                free_slots.append(slot)
                del running[slot]
        while pending and free_slots and (not realtime or pending[0]["arrival"] <= now):
            job = pending[0]
            job["est"] = footprint(job["kind"], job["n"])
            if running and reserved + job["est"] > budget:
                break                          # wait for memory to free up
            pending.popleft()
            slot = free_slots.pop()
            running[slot] = (job, launch(job, slot))
            reserved += job["est"]
            admit_t[job["row"]] = clock()
            max_running = max(max_running, len(running))
    return admit_t, done_t, max_running


class Server:
    def __init__(self, g: Gallatin, slots=32, budget_bytes=None):
        import torch
        self.torch = torch
        self.g = g
        self.slots = slots
        self.streams = [torch.cuda.Stream() for _ in range(slots)]
        self.budget = budget_bytes if budget_bytes is not None else int(0.85 * g.arena_bytes)

    def _launch(self, job, row, results, hist, stream):
        rc = lib().gal_job_launch(self.g.handle, job["kind"], job["id"], job["n"],
                                  C.c_void_p(results[row].data_ptr()),
                                  C.c_void_p(hist.data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != GAL_OK:
            raise GalError(f"gal_job_launch failed ({rc})")

    def run(self, jobs, realtime=True):
        torch = self.torch
        nj = len(jobs)
        results = torch.zeros((nj, 3), dtype=torch.int64, device="cuda")
        hist = torch.zeros(2 * LAT_BINS, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        jobs = [dict(j, row=r) for r, j in enumerate(jobs)]  # result rows follow the input order
        events = [None] * nj

        def launch(job, slot):
            s = self.streams[slot]
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(s)
            self._launch(job, job["row"], results, hist, s)
            end.record(s)
            events[job["row"]] = (start, end)
            return end

        t0 = time.perf_counter()
        admit_t, done_t, max_running = schedule(jobs, self.slots, self.budget, launch,
                                                lambda: time.perf_counter() - t0, realtime, limit_s=300.0)
        wall = time.perf_counter() - t0
        torch.cuda.synchronize()
        res = results.cpu().numpy()
        h = hist.cpu().numpy()
        mh, fh = h[:LAT_BINS], h[LAT_BINS:]
        arrival = np.array([j["arrival"] for j in jobs])
        job_lat = done_t - (arrival if realtime else admit_t)
        wait = admit_t - arrival if realtime else np.zeros(nj)
        dev_ms = np.array([a.elapsed_time(b) for a, b in events])
        ops = int(res[:, 1].sum())
        return {
            "jobs": nj, "ops": ops, "wall_s": wall, "ops_per_s": ops / wall,
            "failed_mallocs": int(res[:, 2].sum()), "max_concurrent_jobs": max_running,
            "job_latency_ms_p50": float(np.percentile(job_lat, 50) * 1e3),
            "job_latency_ms_p99": float(np.percentile(job_lat, 99) * 1e3),
            "admission_wait_ms_p50": float(np.percentile(wait, 50) * 1e3),
            "admission_wait_ms_p99": float(np.percentile(wait, 99) * 1e3),
            "job_device_ms_p50": float(np.percentile(dev_ms, 50)),
            "job_device_ms_p99": float(np.percentile(dev_ms, 99)),
            "latency_requests": {"mallocs": int(mh.sum()), "frees": int(fh.sum())},
            "malloc_cycles_p50": hist_percentile(mh, 50),
            "malloc_cycles_p99": hist_percentile(mh, 99),
            "free_cycles_p50": hist_percentile(fh, 50),
            "free_cycles_p99": hist_percentile(fh, 99),
            "checksums": res[:, 0].astype(np.uint64), "error_word": self.g.error_word(),
        }

    def solo_check(self, jobs, mixed_checksums):
        """Rerun each job alone (nothing else on the device) and compare with
        mixed_checksums, indexed by job id (make_jobs numbers jobs by row)."""
        mism = []
        for job in jobs:
            out = self.run([dict(job, arrival=0.0)], realtime=False)
            if int(out["checksums"][0]) != int(mixed_checksums[job["id"]]):
                mism.append(job["id"])
        return mism


def serve(num_jobs=400, arena_bytes=32 << 30, slots=32, rate=2000.0, seed=5, **cfg):
    g = Gallatin.generate_on_device(arena_bytes, 42, **cfg)
    try:
        srv = Server(g, slots=slots)
        out = srv.run(make_jobs(num_jobs, rate=rate, seed=seed))
        out.pop("checksums")
        out.update(arena_bytes=arena_bytes, slots=slots, rate=rate)
        return out
    finally:
        g.close()
