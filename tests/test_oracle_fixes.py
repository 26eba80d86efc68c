"""The reference defects the product fixes, shown on the CPU oracle.

Leftover credit (block.cuh:267-281): a malloc whose run of slices crosses the
end of its block credits the slices it could not use to the block's free
counter with a plain atomicAdd, on the comment's premise that some slice of the
block is still live.  When every other slice has been freed, that credit is
the one that completes the block, and the reference never returns it.
"""
import numpy as np
import pytest

from gallatin_gb300._abi import FAIL
from oracle.oracle import (FIX_GATHER_EXIT_ROLLBACK, FIX_LEFTOVER_COMPLETES, PRODUCT_FIXES,
                           Oracle, gen_leftover_trace)

# (max_size, slice size of the largest class): one block per segment, and four
GEOMETRIES = [(4096, 4096), (1024, 1024)]


@pytest.mark.parametrize("max_size,slice_size", GEOMETRIES)
def test_leftover_credit_leaks_block_in_reference(max_size, slice_size):
    ops = gen_leftover_trace(slice_size)
    ref = Oracle(1 << 30, 5, max_size=max_size, fixes=FIX_GATHER_EXIT_ROLLBACK)
    out = ref.replay(ops)
    assert (out[:4095] != FAIL).all() and out[-2] != FAIL
    fc = ref.export().free_counters
    leaked = np.flatnonzero(fc == 4096)
    assert len(leaked) == 1, "the reference keeps the completed block's count at 4096"


@pytest.mark.parametrize("max_size,slice_size", GEOMETRIES)
def test_leftover_credit_returns_block_with_fix(max_size, slice_size):
    ops = gen_leftover_trace(slice_size)
    ref = Oracle(1 << 30, 5, max_size=max_size, fixes=FIX_GATHER_EXIT_ROLLBACK)
    fixed = Oracle(1 << 30, 5, max_size=max_size, fixes=PRODUCT_FIXES)
    out_ref, out_fix = ref.replay(ops), fixed.replay(ops)
    assert (out_fix[:4095] == out_ref[:4095]).all()
    assert out_fix[-2] != FAIL
    sv_ref, sv_fix = ref.export(), fixed.export()
    assert (sv_fix.free_counters < 4096).all()
    # the completed block went back to its segment: one more ring entry (or the
    # whole segment released) than in the reference
    assert sv_fix.diff(sv_ref) != []
    assert PRODUCT_FIXES & FIX_LEFTOVER_COMPLETES
