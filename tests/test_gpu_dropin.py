"""The drop-in boundary at the source level: tests/dropin/dropin_test.cu is user
code written against the reference's API (global_allocator.cuh's
init_global_allocator / global_malloc / global_free / free_global_allocator,
and Gallatin<16 MiB, 16, 4096>::generate_on_device with ->malloc / ->free),
compiled against this library's headers and linked to libgallatin_gb300.so
by build().  It runs the reference's global_test / gallatin_test workload:
every thread allocates, stamps its id, a second kernel checks and frees.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin", "libdropin_test.so")


@pytest.fixture(scope="module")
def D():
    import gallatin_gb300
    gallatin_gb300.lib()
    L = C.CDLL(LIB)
    for f in (L.dropin_global_test, L.dropin_handle_test):
        f.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
        f.restype = C.c_int
    return L


@pytest.mark.parametrize("size", [16, 64, 1000, 4096])
def test_global_api_tid_stamp(D, size):
    out = np.zeros(4, dtype=np.uint64)
    assert D.dropin_global_test(2 << 30, 1 << 20 if size <= 64 else 1 << 18, size, 2, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0]


def test_handle_api_tid_stamp(D):
    out = np.zeros(4, dtype=np.uint64)
    assert D.dropin_handle_test(2 << 30, 1 << 20, 16, 3, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0]


def _fn(D, name, nargs):
    f = getattr(D, name)
    f.argtypes = [C.c_uint64] * nargs + [C.c_void_p]
    f.restype = C.c_int
    return f


def test_host_backed_global_instance(D):
    """init_global_allocator_host / global_malloc_host / global_free_host: the
    allocations live in pinned host memory; the host reads the device's stamps
    through the same pointers."""
    out = np.zeros(4, dtype=np.uint64)
    assert _fn(D, "dropin_host_test", 3)(256 << 20, 1 << 16, 64, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0]


def test_managed_arena_handle(D):
    """Gallatin<...>::generate_on_device_managed: the same tid stamps, read on
    the host through managed memory."""
    out = np.zeros(4, dtype=np.uint64)
    assert _fn(D, "dropin_managed_test", 3)(1 << 30, 1 << 16, 64, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0]


def test_fused_malloc_falls_back_to_host(D):
    """global_malloc_fused: a 512 MiB device arena cannot hold 1 GiB of 4 KiB
    requests, so part of them is served from the host instance; every stamp
    survives and global_free_fused returns each pointer to its owner."""
    out = np.zeros(4, dtype=np.uint64)
    assert _fn(D, "dropin_fused_test", 4)(512 << 20, 2 << 30, 1 << 18, 4096, out.ctypes.data) == 0
    misses, bad, on_host, err = out.tolist()
    assert misses == 0 and bad == 0 and err == 0
    assert 0 < on_host < 1 << 18


def test_poison_detects_padding_writes(D):
    """global_malloc_poison / global_check_poison / global_free_poison: intact
    allocations pass, a byte changed in the padding after the user region is
    reported, the user region is untouched."""
    out = np.zeros(5, dtype=np.uint64)
    assert _fn(D, "dropin_poison_test", 3)(2 << 30, 1 << 14, 100, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0, 0]


def test_concurrent_global_init_installs_one_instance():
    """Host threads racing init_global_allocator: one instance is installed,
    the others get GAL_ERR_STATE and leave nothing behind."""
    import threading

    import gallatin_gb300 as G
    L = G.lib()
    assert L.gal_global() is None
    rcs = []
    lock = threading.Lock()

    def init():
        rc = L.gal_init(1 << 30, 42, None)
        with lock:
            rcs.append(rc)

    threads = [threading.Thread(target=init) for _ in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    try:
        assert sorted(rcs) == [G._abi.GAL_OK] + [G._abi.GAL_ERR_STATE] * 3
        assert L.gal_global() is not None
    finally:
        assert L.gal_teardown() == G._abi.GAL_OK
    assert L.gal_global() is None


@pytest.mark.parametrize("n,rounds,lo,hi,arena", [
    (1 << 20, 16, 16, 4096, 8 << 30),        # slices of every class
    (1 << 16, 16, 16, 64 << 10, 8 << 30),    # plus big slices and whole blocks
], ids=["slices", "blocks"])
def test_pointer_churn_exchange_check(D, n, rounds, lo, hi, arena):
    """The reference's global_churn: malloc, exchange the id in and out, free,
    in a loop per thread; no allocation is ever shared and none fails."""
    D.dropin_churn_test.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_uint64, C.c_uint64, C.c_void_p]
    D.dropin_churn_test.restype = C.c_int
    out = np.zeros(4, dtype=np.uint64)
    assert D.dropin_churn_test(arena, n, rounds, lo, hi, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 0]


@pytest.mark.parametrize("calloc_mode", [1, 0], ids=["calloc", "plain"])
def test_calloc_mode_hands_out_zeroed_memory(D, calloc_mode):
    """running_calloc = true: every allocation reads zero, also on memory that
    earlier rounds wrote and freed.  Without it the same rounds do see that
    memory again (the check detects dirt), the reference's plain behaviour."""
    D.dropin_calloc_test.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_void_p]
    D.dropin_calloc_test.restype = C.c_int
    out = np.zeros(4, dtype=np.uint64)
    assert D.dropin_calloc_test(4 << 30, 1 << 14, 6, calloc_mode, out.ctypes.data) == 0
    assert out[0] == 0 and out[3] == 0
    if calloc_mode:
        assert out[1] == 0
    else:
        assert out[1] > 0


def test_unset_global_handle_returns_null(D):
    """A global handle that was never set in the caller's translation unit, or
    was cleared by free_global_allocator, gives nullptr from global_malloc (and
    from the host and poison variants) and a global_free that does nothing;
    between the two, the initialised instance serves."""
    D.dropin_null_handle_test.argtypes = [C.c_uint64, C.c_void_p]
    D.dropin_null_handle_test.restype = C.c_int
    out = np.zeros(5, dtype=np.uint64)
    assert D.dropin_null_handle_test(4096, out.ctypes.data) == 0
    assert out.tolist() == [0, 0, 0, 1, 0]
