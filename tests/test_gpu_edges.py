"""Edge cases of the request sizes and of the calling pattern.

* Sizes at every tier boundary (0 and 1 byte, the slice classes' edges, the
  4-32 KiB runs of 4 KiB slices, whole blocks up to one segment, multi-segment
  runs, and more than the arena) replayed by one device thread: offsets and
  the whole state equal the oracle's; a request larger than the arena returns
  null without setting an error.
* Null entries in the per-thread free are skipped; a zero-byte request gets
  the smallest slice.
* Device code that calls malloc/free divergently, in data-dependent loops with
  early exits (tests/dropin/dropin_test.cu `dropin_divergent_test`), keeps
  every allocation intact and leaves no error.
"""
import ctypes as C
import os

import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import PRODUCT_FIXES, Oracle

pytestmark = pytest.mark.gpu

MIB = 1 << 20
EDGE_SIZES = [0, 1, 15, 16, 17, 31, 32, 33, 2048, 2049, 4095, 4096, 4097, 8191, 8192, 8193, 32767,
              32768, 32769, 65536, 65537, MIB, 16 * MIB - 1, 16 * MIB, 16 * MIB + 1, 48 * MIB,
              100 * MIB, 1 << 40]


@pytest.fixture(scope="module")
def G():
    import gallatin_gb300
    return gallatin_gb300


def _edge_trace():
    ops = []
    for rep in range(3):
        start = len(ops)
        ops += EDGE_SIZES
        # free every other one of this pass, newest first
        ops += [(1 << 63) | i for i in range(len(ops) - 1, start - 1, -2)]
    return np.array(ops, dtype=np.uint64)


@pytest.mark.parametrize("nbytes", [1 << 30, 4 << 30])
def test_edge_sizes_match_oracle(G, nbytes):
    ops = _edge_trace()
    g = G.Gallatin.generate_on_device(nbytes, 42)
    try:
        out, smid = g.replay(ops)
        o = Oracle(nbytes, 42, fixes=PRODUCT_FIXES)
        np.testing.assert_array_equal(out, o.replay(ops, smid=smid))
        assert g.export().diff(o.export()) == []
        assert g.error_word() == 0, g.error_info()
        mallocs = out[ops < (1 << 63)]
        assert mallocs[len(EDGE_SIZES) - 1] == FAIL   # more than the arena: null
        assert mallocs[0] != FAIL                       # zero bytes: the smallest slice
    finally:
        g.close()


def test_zero_bytes_and_null_frees(G):
    import torch
    g = G.Gallatin.generate_on_device(1 << 30, 42)
    try:
        sizes = torch.tensor([0, 1, 16, 0, 1 << 40], dtype=torch.int64, device="cuda")
        ptrs = torch.zeros(5, dtype=torch.int64, device="cuda")
        g.malloc_per_thread(sizes, ptrs)
        torch.cuda.synchronize()
        p = ptrs.cpu().numpy()
        assert (p[:4] != 0).all() and p[4] == 0
        assert len(set(p[:4].tolist())) == 4
        g.free_per_thread(ptrs)           # the null entry is skipped
        g.free_per_thread(torch.zeros(8, dtype=torch.int64, device="cuda"))
        torch.cuda.synchronize()
        assert g.error_word() == 0, g.error_info()
    finally:
        g.close()


def test_divergent_calls_in_loops(G):
    G.lib()
    lib = C.CDLL(os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin", "libdropin_test.so"))
    f = lib.dropin_divergent_test
    f.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
    f.restype = C.c_int
    out = np.zeros(4, dtype=np.uint64)
    assert f(4 << 30, 1 << 16, 3, out.ctypes.data) == 0
    allocs, bad, overlaps, err = out.tolist()
    assert allocs > 0
    assert bad == 0 and overlaps == 0 and err == 0
