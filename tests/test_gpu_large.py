"""Large and block-size allocations on a 64 GiB arena (the vEB over 4,096
segments has three layers): fill to 70%, 10 rounds of freeing 30% and
refilling, every live range checked for overlap and tier alignment after each
round, multi-segment runs all returned after the drain, error word clear."""
import pytest

pytestmark = pytest.mark.gpu


def test_large_block_workload_64GiB():
    import gallatin_gb300 as G
    from gallatin_gb300.workloads import large_block_workload
    g = G.Gallatin.generate_on_device(64 << 30, 7)
    try:
        assert g.dims().veb_layers == 3
        st = large_block_workload(g)
        assert st["overlaps"] == 0 and st["misaligned"] == 0, st
        assert st["error_word"] == 0, (st, g.error_info())
        assert st["multi_segment_allocs_after_drain"] == 0
        assert st["mallocs"] > 20000 and st["frees"] == st["mallocs"]
        assert all(0 < f <= 1 for f in st["fragmentation"])
    finally:
        g.close()
