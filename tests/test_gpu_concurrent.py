"""Concurrent correctness of the CUDA allocator on the GPU (through the C ABI).

Invariants (no reference counterpart gives exact offsets here):
  * every live allocation is non-null, aligned to its size class inside a
    16 MiB-aligned segment, and no two live ranges overlap;
  * stamped payloads read back intact (the reference's tid-stamp test and its
    exchange-check churn, tests/src/global_test.cu, global_churn.cu);
  * the device error word stays clear;
  * a full drain leaves every block's counters balanced.
"""
import numpy as np
import pytest

from gallatin_gb300._abi import GAL_DEV_ERR_BAD_FREE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import gallatin_gb300
    return gallatin_gb300


@pytest.fixture(scope="module")
def torch():
    import torch as t
    return t


SEG = 16 << 20


def _class_bytes(sizes):
    """Bytes a request occupies (Gallatin::get_allocated_size, gallatin.cuh:1152)."""
    s = np.maximum(sizes, 16)
    c = 1 << np.ceil(np.log2(s)).astype(np.int64)
    big = s > SEG
    c[big] = ((s[big] - 1) // SEG + 1) * SEG
    return c


def _alignment(sizes):
    """Slices: their size; 8-32 KiB (runs of 4 KiB slices): 4 KiB; whole blocks:
    the block size; segment runs: 16 MiB."""
    c = _class_bytes(sizes)
    a = c.copy()
    a[(sizes > 4096) & (sizes <= 32768)] = 4096
    a[sizes > SEG] = SEG
    return a


def _check_no_overlap(ptrs, sizes, base):
    order = np.argsort(ptrs)
    p, n, a = ptrs[order], _class_bytes(sizes)[order], _alignment(sizes)[order]
    assert (p[1:] >= p[:-1] + n[:-1]).all(), "live allocations overlap"
    assert (((p - base) % a) == 0).all(), "misaligned allocation"


def test_stamp_1m_threads_16B(G):
    """Config-1 concurrent case: 1,048,576 threads x malloc(16), tid stamp, check, free."""
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        ms, st = g.bench_stamp(1 << 20, 16, rounds=3)
        assert st[0] == 3 << 20 and st[1] == 0, st
        assert st[2] == 0 and st[3] == 3 << 20, st
        assert g.error_word() == 0, g.error_info()
    finally:
        g.close()


@pytest.mark.parametrize("batched", [False, True])
def test_mixed_sizes_no_overlap(G, torch, batched):
    n = 1 << 20
    rng = np.random.default_rng(1 if batched else 2)
    sizes = (2 ** rng.uniform(4, 12, n)).astype(np.int64)
    g = G.Gallatin.generate_on_device(4 << 30, 42)
    try:
        d_sizes = torch.from_numpy(sizes).cuda()
        d_ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        (g.malloc_batched if batched else g.malloc_per_thread)(d_sizes, d_ptrs)
        torch.cuda.synchronize()
        ptrs = d_ptrs.cpu().numpy()
        assert (ptrs != 0).all()
        _check_no_overlap(ptrs, sizes, g.arena_base)
        (g.free_batched if batched else g.free_per_thread)(d_ptrs)
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
        sv = g.export()
        # every counted free matched a claimed slice: no free counter above 4096
        assert (sv.free_counters <= 4096).all()
    finally:
        g.close()


def test_block_and_segment_tiers_no_overlap(G, torch):
    n = 4096
    rng = np.random.default_rng(3)
    sizes = (2 ** rng.uniform(13, 27, n)).astype(np.int64)  # 8 KiB .. 128 MiB
    sizes[sizes > (64 << 20)] = 40 << 20
    g = G.Gallatin.generate_on_device(64 << 30, 7)
    try:
        d_sizes = torch.from_numpy(sizes).cuda()
        d_ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(d_sizes, d_ptrs)
        torch.cuda.synchronize()
        ptrs = d_ptrs.cpu().numpy()
        ok = ptrs != 0
        assert ok.mean() > 0.5
        _check_no_overlap(ptrs[ok], sizes[ok], g.arena_base)
        g.free_per_thread(d_ptrs)
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
        st = g.stats()
        assert st.multi_segment_allocs == 0
    finally:
        g.close()


@pytest.mark.parametrize("batched", [False, True])
def test_churn_payloads(G, batched):
    """Mixed 16 B - 4 KiB churn, 50% random frees per round, payload checked."""
    g = G.Gallatin.generate_on_device(16 << 30, 42)
    try:
        N, R = 1 << 18, 6
        ms, r = g.bench_churn(N, R, 1, batched, batched, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0
        assert r.frees == r.mallocs_ok
        assert r.error_word == 0
    finally:
        g.close()


@pytest.mark.parametrize("spares,graph", [(0, False), (1, False), (1, True)])
def test_churn_e2e_payloads(G, torch, spares, graph):
    """The same churn through the public batched entry points, sizes copied
    from pinned host memory every round (and the step captured as a graph)."""
    g = G.Gallatin.generate_on_device(16 << 30, 42, spare_blocks=spares)
    try:
        N, R = 1 << 18, 4
        sizes = torch.empty(N * R, dtype=torch.int64, pin_memory=True)
        sizes.numpy()[:] = G.churn_sizes(0, N * R, 1).view(np.int64)
        ms, r = g.bench_churn_e2e(sizes.data_ptr(), N, R, 1, 1, 2, use_graph=graph)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0
        assert r.frees == r.mallocs_ok
        assert r.error_word == 0
    finally:
        g.close()


def test_free_batched_n_stops_at_device_count(G, torch):
    """gal_free_batched_n frees exactly the first *d_count entries: the rest of
    the list (the odd half) is freed afterwards by gal_free_batched, which
    would be a double free had the count been ignored."""
    n = 1 << 18
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        sizes = torch.full((n,), 64, dtype=torch.int64, device="cuda")
        ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        g.malloc_batched(sizes, ptrs)
        even, odd = ptrs[0::2].contiguous(), ptrs[1::2].contiguous()
        lst = torch.cat([even, odd])
        cnt = torch.tensor([even.numel()], dtype=torch.int64, device="cuda")
        g.free_batched_n(lst, cnt)
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
        g.free_batched(odd)
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
        sv = g.export()
        assert (sv.free_counters <= 4096).all()
    finally:
        g.close()


TREE_FIELDS = ["seg_tree_words", "sub_tree_words", "tree_ids", "slots", "free_counters"]


@pytest.mark.parametrize("batched", [False, True])
def test_everything_freed_then_trim_gives_fresh_trees(G, torch, batched):
    """Concurrent mixed slice, block and segment requests, all freed, then
    gal_trim: the vEB trees, segment classes, pinned slots and free counters
    are word for word those of a freshly created allocator."""
    n = 1 << 18
    rng = np.random.default_rng(11)
    sizes = (2 ** rng.uniform(4, 12, n)).astype(np.int64)
    sizes[::997] = (2 ** rng.uniform(13, 26, sizes[::997].size)).astype(np.int64)
    g = G.Gallatin.generate_on_device(16 << 30, 42)
    try:
        fresh = g.export()
        d_sizes = torch.from_numpy(sizes).cuda()
        d_ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        (g.malloc_batched if batched else g.malloc_per_thread)(d_sizes, d_ptrs)
        torch.cuda.synchronize()
        assert (d_ptrs.cpu().numpy() != 0).all()
        (g.free_batched if batched else g.free_per_thread)(d_ptrs)
        torch.cuda.synchronize()
        g.trim()
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()


@pytest.mark.parametrize("spares", [0, 1])
def test_churn_then_trim_gives_fresh_trees(G, spares):
    """The batched churn drains every allocation; after trim nothing of it
    remains, the spare blocks prepared by the service warps included."""
    g = G.Gallatin.generate_on_device(16 << 30, 42, spare_blocks=spares)
    try:
        fresh = g.export()
        ms, r = g.bench_churn(1 << 18, 4, 1, True, True, 0, 1)
        assert r.frees == r.mallocs_ok and r.error_word == 0 and r.payload_mismatch == 0
        g.trim()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()


@pytest.mark.parametrize("mode", [1, 1 | (1 << 4), 1 | (2 << 4), 3])
def test_churn_spare_blocks_and_requests_per_thread(G, mode):
    """Spare blocks on, 1, 2 or 4 requests per thread per CTA iteration, and
    the CTA-hash free: the same payload and accounting invariants, per-SM
    slots and 64 MiB segments as in the headline step."""
    g = G.Gallatin.generate_on_device(32 << 30, 42, spare_blocks=1, pinned_slots_first=0,
                                      bytes_per_segment=64 << 20, gather_unlocked_below=16)
    try:
        N, R = 1 << 19, 6
        ms, r = g.bench_churn(N, R, 1, mode, True, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0
        assert r.frees == r.mallocs_ok
        assert r.error_word == 0
    finally:
        g.close()


def test_churn_rounds_must_align(G):
    """Rounds are whole warps of liveness words: a round size that is not a
    multiple of 128 requests is refused before anything launches."""
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        with pytest.raises(G.GalError):
            g.bench_churn(1000, 2, 1, True, True, 0, 1)
    finally:
        g.close()


def test_batch_larger_than_the_arena(G, torch):
    """gal_malloc_batched asked for more than the arena holds: the requests
    it cannot serve come back as nullptr, the rest are disjoint, and freeing
    them gives the segments back."""
    g = G.Gallatin.generate_on_device(512 << 20, 42)
    try:
        n = 300_000
        d_sizes = torch.full((n,), 4096, dtype=torch.int64, device="cuda")
        d_sizes[::3] = 64
        d_ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        g.malloc_batched(d_sizes, d_ptrs)
        torch.cuda.synchronize()
        ptrs = d_ptrs.cpu().numpy()
        sizes = d_sizes.cpu().numpy()
        ok = ptrs != 0
        assert 0 < ok.sum() < n
        _check_no_overlap(ptrs[ok], sizes[ok], g.arena_base)
        assert g.error_word() == 0, g.error_info()
        g.free_batched(d_ptrs)
        torch.cuda.synchronize()
        assert g.stats().free_segments > 0
        assert g.error_word() == 0, g.error_info()
        assert (g.export().free_counters <= 4096).all()
    finally:
        g.close()


def test_exhaustion_returns_null_then_recovers(G, torch):
    """Tiny arena: 4 KiB class runs dry, frees give whole segments back, and
    whole-block requests are served again."""
    g = G.Gallatin.generate_on_device(512 << 20, 42)
    try:
        n = 200_000
        d_sizes = torch.full((n,), 4096, dtype=torch.int64, device="cuda")
        d_ptrs = torch.zeros(n, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(d_sizes, d_ptrs)
        torch.cuda.synchronize()
        ptrs = d_ptrs.cpu().numpy()
        got = (ptrs != 0).sum()
        assert 0 < got < n                     # ran out of memory, returned nullptr
        _check_no_overlap(ptrs[ptrs != 0], np.full(got, 4096), g.arena_base)
        assert g.error_word() == 0, g.error_info()
        g.free_per_thread(d_ptrs)
        torch.cuda.synchronize()
        st = g.stats()
        assert st.free_segments > 0
        big = torch.full((8,), 8 << 20, dtype=torch.int64, device="cuda")
        bp = torch.zeros(8, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(big, bp)
        torch.cuda.synchronize()
        assert (bp.cpu().numpy() != 0).sum() >= 1
        g.free_per_thread(bp)
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
    finally:
        g.close()


def test_double_free_is_reported_not_trapped(G, torch):
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        big = torch.full((1,), 20 << 20, dtype=torch.int64, device="cuda")
        bp = torch.zeros(1, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(big, bp)
        g.free_per_thread(bp)
        g.free_per_thread(bp)  # second free of a multi-segment run
        torch.cuda.synchronize()
        assert g.error_word() & GAL_DEV_ERR_BAD_FREE
        g.clear_error()
        assert g.error_word() == 0, g.error_info()
    finally:
        g.close()


def test_wait_on_a_lock_nobody_releases_times_out(G, torch):
    """Failure detection without a GPU fault: a class lock that nothing will
    release (set through the state import) makes the segment gather's bounded
    wait give up.  The request returns null, the error word carries TIMEOUT,
    the context stays usable, and the same request succeeds once the lock is
    released."""
    from gallatin_gb300._abi import GAL_DEV_ERR_TIMEOUT
    g = G.Gallatin.generate_on_device(1 << 30, 42, spin_limit=64, gather_unlocked_below=0)
    try:
        sv = g.export()
        sv.locks = 0x3FF                   # every class lock and the run lock held
        g.load(sv)
        # two whole 16 MiB blocks of the largest class: the segment gathered
        # ahead at boot serves one, the other needs a gather behind the lock
        sizes = torch.full((2,), 16 << 20, dtype=torch.int64, device="cuda")
        ptrs = torch.zeros(2, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(sizes, ptrs)
        torch.cuda.synchronize()
        p = ptrs.cpu().numpy()
        assert (p != 0).sum() == 1
        assert g.error_word() & GAL_DEV_ERR_TIMEOUT
        g.free_per_thread(ptrs)
        sv = g.export()
        sv.locks = 0
        g.load(sv)
        g.clear_error()
        one = torch.full((1,), 16 << 20, dtype=torch.int64, device="cuda")
        got = torch.zeros(1, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(one, got)
        torch.cuda.synchronize()
        assert int(got.cpu()[0]) != 0
        assert g.error_word() == 0, g.error_info()
        g.free_per_thread(got)
        torch.cuda.synchronize()
    finally:
        g.close()


@pytest.mark.parametrize("mode", [4, 4 | 128, 4 | 8, 8, 4 | 64, 8 | 64])
def test_cached_block_churn_payloads_and_fresh_trees(G, mode):
    """Mallocs from persistent CTAs that cache their SM's pinned blocks in
    shared memory (2 and 4 CTAs per SM), the allocator-only forms without
    payloads, and the free phase with and without the segment classes staged
    in shared memory: every malloc served, payloads intact, frees balance the
    mallocs, and after trim the trees are fresh again."""
    g = G.Gallatin.generate_on_device(32 << 30, 42, spare_blocks=1, pinned_slots_first=0,
                                      bytes_per_segment=64 << 20, gather_unlocked_below=16)
    try:
        fresh = g.export()
        N, R = 1 << 19, 6
        ms, r = g.bench_churn(N, R, 1, mode, True, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0
        assert r.frees == r.mallocs_ok
        assert r.error_word == 0
        g.trim()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()


@pytest.mark.parametrize("mode", [256, 128 | 512, 256 | 512, 8 | 256 | 512])
def test_per_thread_churn_forms_payloads_and_fresh_trees(G, mode):
    """The per-thread malloc kernel compiled for 3 or 4 CTAs per SM and the
    free kernel compiled for 4 CTAs per SM, with and without payloads: every
    malloc served, payloads intact, frees balance the mallocs, and after trim
    the trees are fresh again."""
    g = G.Gallatin.generate_on_device(32 << 30, 42, spare_blocks=1, pinned_slots_first=0,
                                      bytes_per_segment=64 << 20, gather_unlocked_below=16)
    try:
        fresh = g.export()
        N, R = 1 << 19, 6
        ms, r = g.bench_churn(N, R, 1, mode, True, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0
        assert r.frees == r.mallocs_ok
        assert r.error_word == 0
        g.trim()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()


@pytest.mark.parametrize("layout", [0, 1])
def test_block_layouts_serve_the_same_churn(G, layout):
    """Dense counter arrays and one 32-byte record per block: the same churn,
    the same invariants."""
    g = G.Gallatin.generate_on_device(16 << 30, 42, block_layout=layout)
    try:
        N, R = 1 << 18, 6
        ms, r = g.bench_churn(N, R, 1, 4, True, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0 and r.frees == r.mallocs_ok and r.error_word == 0
    finally:
        g.close()


@pytest.mark.parametrize("spares", [0, 1])
def test_exhausted_block_left_in_a_slot_is_replaced(G, torch, spares):
    """A pinned slot that holds a block whose slices are all handed out, with
    no claim left to cross its end (what a stale claim on a recycled block can
    leave behind), is replaced by the next team that finds it there twice:
    the request is served from a new block and nothing is reported."""
    g = G.Gallatin.generate_on_device(2 << 30, 42, spare_blocks=spares, smid_override=0)
    try:
        sv = g.export()
        blk = int(sv.slots_of(0)[0])            # the block pinned in class 0, slot 0
        # exhausted long ago: every slice handed out and many claims failed since
        sv.malloc_counters[blk] = (0 << 20) | (4096 + (1 << 12))
        g.load(sv)
        sizes = torch.full((1,), 16, dtype=torch.int64, device="cuda")
        ptrs = torch.zeros(1, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(sizes, ptrs)
        torch.cuda.synchronize()
        assert int(ptrs.item()) != 0
        after = g.export()
        assert int(after.slots_of(0)[0]) != blk
        assert g.error_word() == 0, g.error_info()
    finally:
        g.close()


@pytest.mark.parametrize("knobs", [dict(l2_fetch_bytes=32), dict(gather_ahead=0), dict(l2_fetch_bytes=64, gather_ahead=0)])
def test_context_hint_and_on_demand_gathers_serve_the_churn(G, knobs):
    """The L2 fetch hint set at create time and segments gathered only on
    demand leave the results alone: every malloc served, payloads intact,
    counts balanced, fresh trees after trim."""
    g = G.Gallatin.generate_on_device(32 << 30, 42, spare_blocks=1, pinned_slots_first=0,
                                      bytes_per_segment=64 << 20, gather_unlocked_below=16, **knobs)
    try:
        fresh = g.export()
        N, R = 1 << 19, 6
        ms, r = g.bench_churn(N, R, 1, 256 | 512, True, 1, 2)
        assert r.mallocs_ok == 2 * N * R and r.mallocs_failed == 0
        assert r.payload_mismatch == 0 and r.frees == r.mallocs_ok and r.error_word == 0
        g.trim()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()
