"""Chained hash tables served by the allocator (gallatin_gb300/csrc/gal_tables.cu).

Insert all, delete a random half (empty nodes unlinked and freed), reinsert:
every key is found with its value after each phase, deleted keys are absent,
each table's live count is its size, every node goes back to the allocator at
teardown, and one table's contents equal the host's copy of the same keys
(the host check of the table's own dict).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TREE_FIELDS = ["seg_tree_words", "sub_tree_words", "tree_ids", "slots", "free_counters"]


@pytest.fixture(scope="module")
def G():
    import gallatin_gb300
    return gallatin_gb300


@pytest.fixture(scope="module")
def T():
    from gallatin_gb300 import tables
    return tables


@pytest.mark.parametrize("batched,width", [(False, 32), (True, 32), (True, 8)])
def test_tables_insert_delete_reinsert(G, T, batched, width):
    sizes = T.table_sizes(64, 8, 13, seed=3)
    g = G.Gallatin.generate_on_device(4 << 30, 42, team_width=width)
    try:
        fresh = g.export()
        d = T.run(g, sizes, seed=3, batched=batched, dump_table=5)
        n = int(sizes.sum())
        assert d["violations"] == 0, d
        assert d["total_pairs"] == n
        assert 0.4 * n < d["deleted"] < 0.6 * n
        assert d["inserted"] == n + d["deleted"]
        # every node came back: deletes of emptied nodes, spares, teardown
        assert d["nodes_allocated"] == d["nodes_freed"] + d["spare_nodes_freed"]
        keys, vals = d["dump"]
        want = T.table_keys(5, int(sizes[5]), seed=3)
        order = np.argsort(keys)
        np.testing.assert_array_equal(keys[order], np.sort(want))
        np.testing.assert_array_equal(vals[order], T.table_values(keys[order]))
        # nothing of the tables is left: after trim the trees are fresh
        g.trim()
        assert g.error_word() == 0, g.error_info()
        assert g.export().diff(fresh, fields=TREE_FIELDS) == []
    finally:
        g.close()


def test_tables_coins_match_host(G, T):
    """The delete coins the device used are the host's: the count deleted is
    the host's count of set coins."""
    sizes = T.table_sizes(16, 8, 11, seed=9)
    g = G.Gallatin.generate_on_device(2 << 30, 42)
    try:
        d = T.run(g, sizes, seed=9, batched=True)
        want = sum(int(T.table_coins(T.table_keys(t, int(n), seed=9)).sum()) for t, n in enumerate(sizes))
        assert d["deleted"] == want
        assert d["violations"] == 0
    finally:
        g.close()
