"""The autotuner's search grid keeps only geometries the reference accepts
(bytes_per_segment >= max_size * 4096, gallatin.cuh:300)."""
import numpy as np

from gallatin_gb300 import autotune


def test_grid_is_legal_and_complete():
    g = list(autotune.grid())
    assert g, "empty grid"
    for k in g:
        assert (k["segment_mib"] << 20) >= k["max_size"] * 4096
    geoms = {(k["segment_mib"], k["min_size"], k["max_size"]) for k in g}
    assert geoms == {(16, 16, 4096), (16, 128, 4096), (64, 16, 4096), (64, 128, 4096),
                     (64, 16, 16384), (64, 128, 16384)}
    assert {k["form"] for k in g} == set(autotune.FORM_MODES)
    assert len(g) == len({tuple(sorted(k.items())) for k in g})


def test_tables_grid_is_the_legal_part_of_the_search_space():
    from gallatin_gb300 import tables
    pts = list(tables.grid())
    assert len(pts) == 18
    for p in pts:
        assert (p["segment_mib"] << 20) >= p["max_size"] * 4096
        assert p["team_width"] in (8, 16, 32)
    assert not any(p["segment_mib"] == 4 for p in pts)


def test_tables_sizes_and_keys():
    from gallatin_gb300 import tables
    s = tables.table_sizes(512, 12, 22, seed=3)
    assert s.min() >= 1 << 12 and s.max() <= 1 << 22
    k = tables.table_keys(7, 100000, seed=3)
    assert len(np.unique(k)) == len(k)            # a bijection of distinct inputs
    c = tables.table_coins(k)
    assert 0.48 < c.mean() < 0.52
