"""Further workloads of the allocator beyond the headline churn (bench.py).

large_block_workload: large and block-size allocations (64 GiB arena; requests
log-uniform over 64 KiB–256 MiB, served as whole blocks up to 16 MiB and as
2–16 contiguous 16 MiB segments beyond, interleaved with 64 B slices at 20
per large request).  Fill to 70% of the arena, then 10 rounds of freeing a
random 30% of the live allocations and refilling with fresh sizes.  The arena
holds ~1,400 such requests at once, so a run issues a few thousand large
requests.  Every live allocation is checked for overlap and alignment after
each round; fragmentation = largest run of free segments / free segments.
"""
import numpy as np

SEG = 16 << 20


def serial_trace(seed, nops, malloc_pct=60, quantum=16, steps=256):
    """A one-thread trace in gal_replay_trace's encoding: malloc_pct% mallocs of
    quantum x [1, steps] bytes, the rest free a random live earlier malloc."""
    rng = np.random.default_rng(seed)
    ops = np.zeros(nops, dtype=np.uint64)
    live = []
    for i in range(nops):
        if not live or rng.integers(100) < malloc_pct:
            ops[i] = quantum * (1 + int(rng.integers(steps)))
            live.append(i)
        else:
            j = live.pop(int(rng.integers(len(live))))
            ops[i] = (1 << 63) | j
    return ops


def occupied_bytes(sizes):
    """Bytes each request holds (Gallatin::get_allocated_size, gallatin.cuh:1152)."""
    s = np.maximum(np.asarray(sizes, dtype=np.int64), 16)
    c = 1 << np.ceil(np.log2(s)).astype(np.int64)
    big = s > SEG
    c[big] = ((s[big] - 1) // SEG + 1) * SEG
    return c


def alignment(sizes):
    s = np.asarray(sizes, dtype=np.int64)
    a = occupied_bytes(s)
    a[(s > 4096) & (s <= 32768)] = 4096
    a[s > SEG] = SEG
    return a


def check_live(ptrs, sizes, base):
    """No two live ranges overlap and each pointer has its tier's alignment."""
    order = np.argsort(ptrs)
    p, n, a = ptrs[order], occupied_bytes(sizes)[order], alignment(sizes)[order]
    overlap = int((p[1:] < p[:-1] + n[:-1]).sum())
    misaligned = int((((p - base) % a) != 0).sum())
    return overlap, misaligned


class TorchBackend:
    """large_block_workload's view of this library's allocator: per-thread
    malloc/free calls through the C ABI on device arrays, timed with CUDA
    events around each launch."""

    def __init__(self, g):
        import torch
        self.g = g
        self.arena_bytes = g.arena_bytes
        self.arena_base = g.arena_base
        self._ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))

    def _timed(self, fn, *args):
        ev0, ev1 = self._ev
        ev0.record()
        fn(*args)
        ev1.record()
        ev1.synchronize()
        return ev0.elapsed_time(ev1)

    def malloc(self, sizes):
        import torch
        d_sizes = torch.from_numpy(np.ascontiguousarray(sizes, dtype=np.int64)).cuda()
        d_ptrs = torch.zeros(len(sizes), dtype=torch.int64, device="cuda")
        ms = self._timed(self.g.malloc_per_thread, d_sizes, d_ptrs)
        return d_ptrs.cpu().numpy(), ms

    def free(self, ptrs):
        import torch
        d_ptrs = torch.from_numpy(np.ascontiguousarray(ptrs, dtype=np.int64)).cuda()
        return self._timed(self.g.free_per_thread, d_ptrs)

    def free_runs(self):
        """(largest run of free segments, free segments)"""
        st = self.g.stats()
        return int(st.largest_free_run), int(st.free_segments)

    def extra(self):
        st = self.g.stats()
        return {"multi_segment_allocs_after_drain": int(st.multi_segment_allocs),
                "error_word": self.g.error_word()}


def largest_run_of_ones(words, n):
    """Longest run of set bits among the first n bits of a u64 word array."""
    bits = np.unpackbits(np.ascontiguousarray(words, dtype="<u8").view(np.uint8), bitorder="little")[:n]
    if not bits.any():
        return 0
    edges = np.diff(np.concatenate([[0], bits.astype(np.int8), [0]]))
    return int((np.flatnonzero(edges == -1) - np.flatnonzero(edges == 1)).max())


def large_block_workload(g, seed=3, fill=0.70, rounds=10, small_per_large=20, batch=256,
                         free_frac=0.30):
    """Runs the workload on `g`: a Gallatin (this library) or any backend with
    malloc(sizes) -> (pointers, ms), free(pointers) -> ms, free_runs(),
    extra(), arena_bytes and arena_base."""
    be = g if hasattr(g, "free_runs") else TorchBackend(g)
    rng = np.random.default_rng(seed)
    arena = be.arena_bytes
    target = fill * arena
    live_p = np.zeros(0, dtype=np.int64)
    live_s = np.zeros(0, dtype=np.int64)
    stats = {"mallocs": 0, "frees": 0, "failed": 0, "large_requests": 0, "gpu_ms": 0.0,
             "fragmentation": [], "overlaps": 0, "misaligned": 0}

    def allocate(n_large):
        nonlocal live_p, live_s
        large = (2 ** rng.uniform(16, 28, n_large)).astype(np.int64)
        sizes = np.concatenate([large, np.full(n_large * small_per_large, 64, dtype=np.int64)])
        rng.shuffle(sizes)
        ptrs, ms = be.malloc(sizes)
        ptrs = np.asarray(ptrs).view(np.int64)
        stats["gpu_ms"] += ms
        ok = ptrs != 0
        stats["mallocs"] += int(ok.sum())
        stats["failed"] += int((~ok).sum())
        stats["large_requests"] += n_large
        live_p = np.concatenate([live_p, ptrs[ok]])
        live_s = np.concatenate([live_s, sizes[ok]])
        return int((~ok[sizes > 64]).sum())

    def fill_up():
        while occupied_bytes(live_s).sum() < target:
            if allocate(batch) > batch // 2:      # the arena is as full as it gets
                break

    def round_report():
        o, m = check_live(live_p, live_s, be.arena_base)
        stats["overlaps"] += o
        stats["misaligned"] += m
        run, free = be.free_runs()
        frag = run / free if free else 1.0
        stats["fragmentation"].append(round(float(frag), 4))

    fill_up()
    round_report()
    for _ in range(rounds):
        victims = rng.random(len(live_p)) < free_frac
        stats["gpu_ms"] += be.free(live_p[victims])
        stats["frees"] += int(victims.sum())
        live_p, live_s = live_p[~victims], live_s[~victims]
        fill_up()
        round_report()
    # drain
    stats["gpu_ms"] += be.free(live_p)
    stats["frees"] += len(live_p)
    stats.update(be.extra())
    stats["ops_per_s"] = (stats["mallocs"] + stats["frees"]) / (stats["gpu_ms"] / 1e3)
    stats["live_fraction_target"] = fill
    return stats
