"""gal_export_state_noalloc: the state export for callers that cannot allocate
device memory at that moment (a caching allocator already holds the device's
memory, the snapshot must not wait for the whole device as cudaFree does, or
the device-memory budget is fixed).  It must return exactly what
gal_export_state returns, call after call, without growing device memory use.

Kept in a file collected last, so a failure here comes after every other test
has run; it passes alone in a fresh process too.
"""
import numpy as np
import pytest

from oracle.oracle import gen_serial_trace

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import gallatin_gb300
    return gallatin_gb300


def _same(a, b):
    assert a.diff(b) == [], a.diff(b)
    assert a.error_word == b.error_word


def test_noalloc_export_matches_export_twice_in_a_row(G):
    import torch
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        g.replay(gen_serial_trace(7, 4096, 60, 16, 256))
        first = g.export_noalloc()                  # first call on this device: sets up
        _same(first, g.export())
        g.replay(gen_serial_trace(8, 20000, 55, 16, 256))  # the state moves on
        torch.cuda.synchronize()
        free_before, _ = torch.cuda.mem_get_info()
        second = g.export_noalloc()                 # same array, new contents
        free_after, _ = torch.cuda.mem_get_info()
        _same(second, g.export())
        assert free_after == free_before, "device memory use changed during the call"
        assert second.diff(first) != []             # not the previous call's contents
    finally:
        g.close()


def test_noalloc_export_rejects_allocators_beyond_its_array(G):
    from gallatin_gb300._abi import GAL_ERR_ARGS
    import ctypes as C
    # 17 GiB at 16 MiB segments and 16 B slices: 278,528 blocks > 262,144
    g = G.Gallatin.generate_on_device(17 << 30, 42)
    try:
        sv = G.StateView(g.dims())
        v = sv.cview()
        assert G.lib().gal_export_state_noalloc(g.handle, C.byref(v)) == GAL_ERR_ARGS
    finally:
        g.close()
