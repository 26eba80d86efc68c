"""The autotuner's search grid keeps only geometries the reference accepts
(bytes_per_segment >= max_size * 4096, gallatin.cuh:300)."""
from gallatin_gb300 import autotune


def test_grid_is_legal_and_complete():
    g = list(autotune.grid())
    assert g, "empty grid"
    for k in g:
        assert (k["segment_mib"] << 20) >= k["max_size"] * 4096
    geoms = {(k["segment_mib"], k["min_size"], k["max_size"]) for k in g}
    assert geoms == {(16, 16, 4096), (16, 128, 4096), (64, 16, 4096), (64, 128, 4096),
                     (64, 16, 16384), (64, 128, 16384)}
    assert {k["free_mode"] for k in g} == {"warp", "cta"}
    assert len(g) == len({tuple(sorted(k.items())) for k in g})
