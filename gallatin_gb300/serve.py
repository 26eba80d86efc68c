"""Served request loop over the device allocator (continuous batching).

Jobs arrive as a Poisson process (default mean 2,000 jobs/s, seed 5).  A job is
either a device vector of uint32 grown by push_back to n elements (n
log-uniform over 1K-16M, capacity doubling through the allocator) or a queue
of 32 B nodes with n enqueue/dequeue operations (n log-uniform over 1K-4M);
each runs as one CTA (gal_job_launch) on a stream slot.  The loop keeps every
slot busy: a job that has arrived is admitted as soon as a slot is free and the
arena bytes reserved by running jobs plus its own estimated footprint fit in
the budget, so jobs arriving while others run overlap with them on the device.
Allocator state stays resident on the device across all jobs.

Reported: malloc+free ops/s over the whole run, job latency (completion -
arrival) p50/p99, per-request malloc/free latency p50/p99 in SM cycles
(clock64 around the first calls of each job), failures.  `solo_check` reruns
jobs one at a time and compares their checksums with the mixed run.
"""
import ctypes as C
import time
from collections import deque

import numpy as np

from . import GAL_OK, Gallatin, GalError, lib

JOB_VECTOR, JOB_QUEUE = 0, 1
LAT = 64
SEG = 16 << 20


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
        cap = max(1024, 1 << int(np.ceil(np.log2(max(n, 1)))))
        new, old = 4 * cap, 2 * cap              # bytes of the last two buffers
        r = lambda b: ((b - 1) // SEG + 1) * SEG if b > SEG else 1 << int(np.ceil(np.log2(b)))
        return r(new) + r(old)
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


def schedule(jobs, slots, budget, launch, clock, realtime=True):
    """The admission loop.  jobs: dicts with kind, n, arrival and row.  A job is
    admitted in arrival order once it has arrived (realtime) or at once, as
    soon as a slot is free and the estimated footprints of the running jobs
    plus its own fit in `budget`; a job that does not fit even alone runs
    alone.  launch(job, slot) starts it and returns an object whose query()
    says whether it has finished; clock() gives seconds since the start.
    Returns the admission and completion times per row and the most jobs that
    ran at once."""
    nj = len(jobs)
    pending = deque(sorted(jobs, key=lambda j: j["arrival"]))
    free_slots = list(range(slots))
    running = {}
    reserved = 0
    admit_t, done_t = np.zeros(nj), np.zeros(nj)
    max_running = 0
    while pending or running:
        now = clock()
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

    def _launch(self, job, row, results, lats, stream):
        rc = lib().gal_job_launch(self.g.handle, job["kind"], job["id"], job["n"],
                                  C.c_void_p(results[row].data_ptr()),
                                  C.c_void_p(lats[row].data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != GAL_OK:
            raise GalError(f"gal_job_launch failed ({rc})")

    def run(self, jobs, realtime=True):
        torch = self.torch
        nj = len(jobs)
        results = torch.zeros((nj, 3), dtype=torch.int64, device="cuda")
        lats = torch.zeros((nj, 2 * LAT), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        jobs = [dict(j, row=r) for r, j in enumerate(jobs)]  # result rows follow the input order

        def launch(job, slot):
            s = self.streams[slot]
            self._launch(job, job["row"], results, lats, s)
            ev = torch.cuda.Event()
            ev.record(s)
            return ev

        t0 = time.perf_counter()
        admit_t, done_t, max_running = schedule(jobs, self.slots, self.budget, launch,
                                                lambda: time.perf_counter() - t0, realtime)
        wall = time.perf_counter() - t0
        torch.cuda.synchronize()
        res = results.cpu().numpy()
        lat = lats.cpu().numpy().astype(np.uint32)
        arrival = np.array([j["arrival"] for j in jobs])
        job_lat = done_t - (arrival if realtime else admit_t)
        m_cyc = lat[:, :LAT][lat[:, :LAT] > 0]
        f_cyc = lat[:, LAT:][lat[:, LAT:] > 0]
        ops = int(res[:, 1].sum())
        return {
            "jobs": nj, "ops": ops, "wall_s": wall, "ops_per_s": ops / wall,
            "failed_mallocs": int(res[:, 2].sum()), "max_concurrent_jobs": max_running,
            "job_latency_ms_p50": float(np.percentile(job_lat, 50) * 1e3),
            "job_latency_ms_p99": float(np.percentile(job_lat, 99) * 1e3),
            "malloc_cycles_p50": float(np.percentile(m_cyc, 50)) if len(m_cyc) else None,
            "malloc_cycles_p99": float(np.percentile(m_cyc, 99)) if len(m_cyc) else None,
            "free_cycles_p50": float(np.percentile(f_cyc, 50)) if len(f_cyc) else None,
            "free_cycles_p99": float(np.percentile(f_cyc, 99)) if len(f_cyc) else None,
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
