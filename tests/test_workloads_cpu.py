"""Host helpers of the secondary workloads (gallatin_gb300/workloads.py): the
bytes and alignment each tier gives a request (Gallatin::get_allocated_size,
gallatin.cuh:1152-1183), the live-range checker, the serial trace generator."""
import numpy as np

from gallatin_gb300.workloads import SEG, alignment, check_live, occupied_bytes, serial_trace


def test_occupied_bytes_per_tier():
    sizes = [1, 16, 17, 100, 4096, 4097, 32768, 32769, SEG, SEG + 1, 40 << 20]
    want = [16, 16, 32, 128, 4096, 8192, 32768, 65536, SEG, 2 * SEG, 48 << 20]
    assert occupied_bytes(sizes).tolist() == want


def test_alignment_per_tier():
    sizes = [16, 100, 4096, 5000, 32768, 40000, SEG, 40 << 20]
    want = [16, 128, 4096, 4096, 4096, 65536, SEG, SEG]
    assert alignment(sizes).tolist() == want


def test_check_live_counts_overlaps_and_misalignment():
    base = 1 << 40
    sizes = np.array([64, 64, 4096, 100], dtype=np.int64)
    ok = np.array([base, base + 64, base + 4096, base + 8192], dtype=np.int64)
    assert check_live(ok, sizes, base) == (0, 0)
    overlapping = ok.copy()
    overlapping[1] = base + 32                      # inside the first 64 B slice
    assert check_live(overlapping, sizes, base)[0] == 1
    misaligned = ok.copy()
    misaligned[3] = base + 8192 + 64                # a 128 B class on a 64 B boundary
    assert check_live(misaligned, sizes, base) == (0, 1)


def test_serial_trace_frees_each_earlier_malloc_at_most_once():
    a, b = serial_trace(7, 5000), serial_trace(7, 5000)
    assert (a == b).all()
    freed = set()
    for i, op in enumerate(a.tolist()):
        if op >> 63:
            j = op & ~(1 << 63)
            assert j < i and not (a[j] >> np.uint64(63)) and j not in freed
            freed.add(j)
        else:
            assert op % 16 == 0 and 16 <= op <= 16 * 256
