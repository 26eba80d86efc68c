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
