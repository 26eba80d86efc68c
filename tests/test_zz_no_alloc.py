"""gal_export_state_noalloc: the state export for callers that cannot allocate
device memory at that moment (a caching allocator already holds the device's
memory, or the device-memory budget is fixed) and for monitors that must not
wait for the whole device.  It must return exactly what gal_export_state
returns, call after call, without changing the device's free memory, also on
its first call.

Kept in a file collected last, so a failure here comes after every other test
has run; it passes alone in a fresh process too.
"""
import os
import subprocess
import sys

import pytest

from oracle.oracle import gen_serial_trace

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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
        torch.cuda.synchronize()
        free_before, _ = torch.cuda.mem_get_info()
        first = g.export_noalloc()                  # the handle's first export
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after == free_before, "device memory use changed during the first call"
        _same(first, g.export())
        g.replay(gen_serial_trace(8, 20000, 55, 16, 256))  # the state moves on
        torch.cuda.synchronize()
        free_before, _ = torch.cuda.mem_get_info()
        second = g.export_noalloc()                 # same array, new contents
        free_after, _ = torch.cuda.mem_get_info()
        _same(second, g.export())
        assert free_after == free_before, "device memory use changed during the second call"
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


CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import torch
import gallatin_gb300 as G
from oracle.oracle import gen_serial_trace
torch.cuda.set_device(0)
g = G.Gallatin.generate_on_device(1 << 30, 42)
g.replay(gen_serial_trace(7, 4096, 60, 16, 256))
torch.cuda.synchronize()
free, _ = torch.cuda.mem_get_info()
hold = torch.empty(free - (64 << 20), dtype=torch.uint8, device="cuda")  # all but 64 MiB
torch.cuda.synchronize()
before, _ = torch.cuda.mem_get_info()
snap = g.export_noalloc()             # the process's first export
after, _ = torch.cuda.mem_get_info()
del hold
torch.cuda.empty_cache()
assert after == before, (before, after)
assert snap.diff(g.export()) == [], "differs from gal_export_state"
g.close()
print("first export ok")
"""


def test_first_noalloc_export_while_the_device_memory_is_held():
    """In a fresh process whose caching allocator holds all but 64 MiB of the
    device, the first export (the set-up was done by gal_create) succeeds and
    changes no device memory."""
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "first export ok" in r.stdout
