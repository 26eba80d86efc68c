"""ctypes mirror of include/gallatin_gb300.h (structs and constants).

Shared by the library wrapper (gallatin_gb300) and by the test-side checker;
it holds layouts only, no behaviour.
"""
import ctypes as C

import numpy as np

GAL_OK = 0
GAL_ERR_ARGS = 1
GAL_ERR_CUDA = 2
GAL_ERR_OOM = 3
GAL_ERR_STATE = 4
GAL_ERR_DEVICE = 5

GAL_DEV_ERR_TIMEOUT = 0x1
GAL_DEV_ERR_BAD_FREE = 0x2
GAL_DEV_ERR_NULL_QUEUE = 0x4
GAL_DEV_ERR_SEGMENT_SETUP = 0x8
GAL_DEV_ERR_SLOT_SWAP = 0x10
GAL_DEV_ERR_BLOCK_TREE = 0x20
GAL_DEV_ERR_BOOT = 0x40

GAL_POLICY_REFERENCE = 0
GAL_POLICY_LOWEST = 1
GAL_ARENA_DEVICE, GAL_ARENA_HOST, GAL_ARENA_MANAGED = 0, 1, 2
GAL_BLOCK_LAYOUT_DENSE, GAL_BLOCK_LAYOUT_RECORD = 0, 1

GAL_MAX_TREES = 16
GAL_MAX_VEB_LAYERS = 8

FAIL = (1 << 64) - 1
FREE_BIT = 1 << 63


class GalConfig(C.Structure):
    _fields_ = [
        ("bytes_per_segment", C.c_uint64),
        ("min_size", C.c_uint64),
        ("max_size", C.c_uint64),
        ("smid_override", C.c_int32),
        ("subtree_policy", C.c_uint32),
        ("pinned_slots_first", C.c_uint32),
        ("pinned_slots_min", C.c_uint32),
        ("zero_arena", C.c_uint32),
        ("spin_limit", C.c_uint32),
        ("gather_unlocked_below", C.c_uint32),
        ("team_width", C.c_uint32),
        ("arena_kind", C.c_uint32),
        ("spare_blocks", C.c_uint32),
        ("zero_fill", C.c_uint32),
        ("block_layout", C.c_uint32),
        ("l2_fetch_bytes", C.c_uint32),
        ("gather_ahead", C.c_uint32),
    ]


class GalStats(C.Structure):
    _fields_ = [
        ("num_segments", C.c_uint64),
        ("free_segments", C.c_uint64),
        ("largest_free_run", C.c_uint64),
        ("num_trees", C.c_uint32),
        ("error_word", C.c_uint32),
        ("tree_segments", C.c_uint64 * GAL_MAX_TREES),
        ("tree_listed", C.c_uint64 * GAL_MAX_TREES),
        ("tree_live_blocks", C.c_uint64 * GAL_MAX_TREES),
        ("multi_segment_allocs", C.c_uint64),
        ("multi_segment_segments", C.c_uint64),
        ("metadata_bytes", C.c_uint64),
    ]


class GalStateDims(C.Structure):
    _fields_ = [
        ("num_segments", C.c_uint64),
        ("num_trees", C.c_uint32),
        ("blocks_per_segment", C.c_uint32),
        ("veb_layers", C.c_uint32),
        ("veb_words", C.c_uint32),
        ("total_slots", C.c_uint32),
        ("slot_counts", C.c_uint32 * GAL_MAX_TREES),
    ]


class GalStateViewC(C.Structure):
    _fields_ = [
        ("seg_tree_words", C.c_void_p),
        ("sub_tree_words", C.c_void_p),
        ("tree_ids", C.c_void_p),
        ("active_counts", C.c_void_p),
        ("queue_counters", C.c_void_p),
        ("queue_free_counters", C.c_void_p),
        ("final_queue_free_counters", C.c_void_p),
        ("malloc_counters", C.c_void_p),
        ("free_counters", C.c_void_p),
        ("queues", C.c_void_p),
        ("slots", C.c_void_p),
        ("locks", C.c_uint32),
        ("error_word", C.c_uint32),
    ]


ARRAY_FIELDS = [
    ("seg_tree_words", np.uint64),
    ("sub_tree_words", np.uint64),
    ("tree_ids", np.uint16),
    ("active_counts", np.int32),
    ("queue_counters", np.uint32),
    ("queue_free_counters", np.uint32),
    ("final_queue_free_counters", np.uint32),
    ("malloc_counters", np.uint32),
    ("free_counters", np.uint32),
    ("queues", np.int32),
    ("slots", np.int32),
]


class StateView:
    """Host copy of a whole allocator state as numpy arrays (gal_state_view)."""

    def __init__(self, dims: GalStateDims):
        self.dims = dims
        S = dims.num_segments
        nb = S * dims.blocks_per_segment
        W = dims.veb_words
        T = dims.num_trees
        sizes = {
            "seg_tree_words": W,
            "sub_tree_words": T * W,
            "tree_ids": S,
            "active_counts": S,
            "queue_counters": S,
            "queue_free_counters": S,
            "final_queue_free_counters": S,
            "malloc_counters": nb,
            "free_counters": nb,
            "queues": nb,
            "slots": dims.total_slots,
        }
        for name, dt in ARRAY_FIELDS:
            setattr(self, name, np.zeros(sizes[name], dtype=dt))
        self.locks = 0
        self.error_word = 0

    def cview(self) -> GalStateViewC:
        v = GalStateViewC()
        for name, _ in ARRAY_FIELDS:
            setattr(v, name, getattr(self, name).ctypes.data)
        v.locks = self.locks
        v.error_word = self.error_word
        return v

    def pull(self, v: GalStateViewC):
        self.locks = v.locks
        self.error_word = v.error_word

    def slots_of(self, tree: int) -> np.ndarray:
        counts = list(self.dims.slot_counts)[: self.dims.num_trees]
        o = sum(counts[:tree])
        return self.slots[o:o + counts[tree]]

    def diff(self, other: "StateView", fields=None):
        """Names of the arrays (and scalars) that differ."""
        out = []
        for name, _ in ARRAY_FIELDS:
            if fields is not None and name not in fields:
                continue
            a, b = getattr(self, name), getattr(other, name)
            if a.shape != b.shape or not np.array_equal(a, b):
                out.append(name)
        if fields is None or "locks" in fields:
            if self.locks != other.locks:
                out.append("locks")
        return out

    def to_npz(self, path, **extra):
        arrays = {name: getattr(self, name) for name, _ in ARRAY_FIELDS}
        dims = np.array([self.dims.num_segments, self.dims.num_trees,
                         self.dims.blocks_per_segment, self.dims.veb_layers,
                         self.dims.veb_words, self.dims.total_slots]
                        + list(self.dims.slot_counts), dtype=np.int64)
        np.savez_compressed(path, _dims=dims, _locks=np.array([self.locks]), **arrays, **extra)

    @staticmethod
    def from_npz(path):
        z = np.load(path)
        d = z["_dims"]
        dims = GalStateDims()
        dims.num_segments, dims.num_trees, dims.blocks_per_segment = int(d[0]), int(d[1]), int(d[2])
        dims.veb_layers, dims.veb_words, dims.total_slots = int(d[3]), int(d[4]), int(d[5])
        for i in range(GAL_MAX_TREES):
            dims.slot_counts[i] = int(d[6 + i])
        sv = StateView(dims)
        for name, dt in ARRAY_FIELDS:
            setattr(sv, name, z[name].astype(dt))
        sv.locks = int(z["_locks"][0])
        return sv, z
