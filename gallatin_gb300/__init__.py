"""GB300-native Gallatin-compatible device allocator — Python host mirror.

The product is libgallatin_gb300.so (C ABI, include/gallatin_gb300.h) plus the
header-inline device malloc/free (include/gallatin_gb300/gal_device.cuh and
the drop-in include/gallatin/allocators/).  This module binds the C ABI with
ctypes under the reference's host-side names (gallatin::allocators:
init_global_allocator, free_global_allocator, print_global_stats and
Gallatin<...>::generate_on_device / free_on_device).  Device buffers are
passed as raw pointers (torch tensors' data_ptr() in the tests and bench).

There is no CPU fallback: loading fails loudly if the CUDA library is missing.
"""
import ctypes as C
import os

import numpy as np

from ._abi import (FAIL, FREE_BIT, GAL_OK, GAL_POLICY_LOWEST, GAL_POLICY_REFERENCE, GalConfig,
                   GalStateDims, GalStateViewC, GalStats, StateView)

HERE = os.path.dirname(os.path.abspath(__file__))
# GALLATIN_GB300_LIB points at another build of the library (same C ABI)
LIB_PATH = os.environ.get("GALLATIN_GB300_LIB", os.path.join(HERE, "libgallatin_gb300.so"))

_lib = None


class GalError(RuntimeError):
    pass


class ChurnResult(C.Structure):
    _fields_ = [
        ("ms_total", C.c_double),
        ("ms_malloc_kernels", C.c_double),
        ("ms_free_kernels", C.c_double),
        ("mallocs_ok", C.c_uint64),
        ("mallocs_failed", C.c_uint64),
        ("payload_mismatch", C.c_uint64),
        ("frees", C.c_uint64),
        ("malloc_launches", C.c_uint64),
        ("free_launches", C.c_uint64),
        ("other_launches", C.c_uint64),
        ("h2d_bytes", C.c_uint64),
        ("d2h_bytes", C.c_uint64),
        ("error_word", C.c_uint32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStream(C.Structure):
    """gal_server_stream (gallatin_gb300/csrc/gal_server.cu)."""
    _fields_ = [
        ("requests", C.c_uint64),
        ("lo", C.c_uint32),
        ("hi", C.c_uint32),
        ("log_uniform", C.c_uint32),
        ("keep", C.c_uint32),
    ]


class ServerResult(C.Structure):
    """gal_server_result (gallatin_gb300/csrc/gal_server.cu)."""
    _fields_ = [
        ("ms_total", C.c_double),
        ("mallocs_ok", C.c_uint64),
        ("mallocs_failed", C.c_uint64),
        ("stamp_mismatch", C.c_uint64),
        ("frees", C.c_uint64),
        ("misaligned", C.c_uint64),
        ("not_zeroed", C.c_uint64),
        ("status", C.c_uint32),
        ("error_word", C.c_uint32),
        ("grid", C.c_uint32),
        ("server_ctas", C.c_uint32),
        ("block", C.c_uint32),
        ("graph", C.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TablesResult(C.Structure):
    """gal_tables_result (gallatin_gb300/csrc/gal_tables.cu)."""
    _fields_ = [
        ("ms", C.c_float * 6),
        ("total_pairs", C.c_uint64),
        ("inserted", C.c_uint64),
        ("deleted", C.c_uint64),
        ("nodes_allocated", C.c_uint64),
        ("nodes_freed", C.c_uint64),
        ("spare_nodes_freed", C.c_uint64),
        ("malloc_failed", C.c_uint64),
        ("lock_timeouts", C.c_uint64),
        ("missing", C.c_uint64),
        ("unexpected", C.c_uint64),
        ("wrong_value", C.c_uint64),
        ("count_mismatch", C.c_uint64),
        ("error_word", C.c_uint64),
        ("setup_failed", C.c_uint64),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "ms"}
        d["ms"] = [float(x) for x in self.ms]
        return d


def lib():
    """Load libgallatin_gb300.so (build it with gallatin_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GalError(f"{LIB_PATH} is missing: the CUDA extension was not built "
                       "(python -m gallatin_gb300.build)")
    L = C.CDLL(LIB_PATH)
    vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int32
    sig = {
        "gal_config_default": ([vp], C.c_int),
        "gal_create": ([u64, u64, vp, C.POINTER(vp)], C.c_int),
        "gal_create_unbooted": ([u64, u64, vp, C.POINTER(vp)], C.c_int),
        "gal_destroy": ([vp], C.c_int),
        "gal_device_state": ([vp], vp),
        "gal_handle_of": ([vp], vp),
        "gal_arena_base": ([vp], vp),
        "gal_arena_bytes": ([vp], u64),
        "gal_get_stats": ([vp, vp], C.c_int),
        "gal_print_stats": ([vp], C.c_int),
        "gal_last_error": ([vp, vp], C.c_int),
        "gal_clear_error": ([vp], C.c_int),
        "gal_error_info": ([vp, vp], C.c_int),
        "gal_state_dims_get": ([vp, vp], C.c_int),
        "gal_export_state": ([vp, vp], C.c_int),
        "gal_export_state_noalloc": ([vp, vp], C.c_int),
        "gal_import_state": ([vp, vp], C.c_int),
        "gal_set_smid_override": ([vp, i32], C.c_int),
        "gal_set_policy": ([vp, u32], C.c_int),
        "gal_init": ([u64, u64, vp], C.c_int),
        "gal_teardown": ([], C.c_int),
        "gal_global": ([], vp),
        "gal_replay_trace": ([vp, vp, u64, vp, vp, vp], C.c_int),
        "gal_replay_warp_trace": ([vp, vp, u64, vp, vp, vp], C.c_int),
        "gal_malloc_per_thread": ([vp, vp, u64, vp, vp], C.c_int),
        "gal_free_per_thread": ([vp, vp, u64, vp], C.c_int),
        "gal_malloc_batched": ([vp, vp, u64, vp, vp], C.c_int),
        "gal_free_batched": ([vp, vp, u64, vp], C.c_int),
        "gal_free_batched_n": ([vp, vp, vp, u64, vp], C.c_int),
        "gal_trim": ([vp, vp], C.c_int),
        "gal_bench_churn": ([vp, u64, u32, u32, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp], C.c_int),
        "gal_bench_churn_e2e": ([vp, vp, u64, u32, u32, C.c_int, C.c_int, vp, vp, C.c_int], C.c_int),
        "gal_churn_sizes": ([u64, u64, u32, vp], C.c_int),
        "gal_bench_stamp": ([vp, u64, u64, C.c_int, vp, vp], C.c_int),
        "gal_bench_latency": ([vp, u64, u32, C.c_int, vp, vp], C.c_int),
        "gal_bench_atomic_peak": ([vp, vp], C.c_int),
        "gal_bench_sector_probe": ([u32, u32, vp], C.c_int),
        "gal_bench_server": ([vp, vp, u32, u32, C.c_int, C.c_int, C.c_int, C.c_int, u32, vp, vp], C.c_int),
        "gal_job_launch": ([vp, u32, u64, u64, vp, vp, vp], C.c_int),
        "gal_job_ctas": ([u32, u64], u32),
        "gal_bench_tables": ([vp, u32, vp, u64, C.c_int, vp, u32, vp, vp, u64, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols():
    """Names of the C ABI entry points this module binds."""
    lib()
    return [n for n in dir(_lib) if n.startswith("gal_")]


def _check(rc, what):
    if rc != GAL_OK:
        raise GalError(f"{what} failed with status {rc}")


def default_config(**kw) -> GalConfig:
    cfg = GalConfig()
    _check(lib().gal_config_default(C.byref(cfg)), "gal_config_default")
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def _ptr(x):
    """Device pointer of a torch tensor (or an int)."""
    return x if isinstance(x, int) else x.data_ptr()


class Gallatin:
    """One allocator instance (Gallatin<bytes_per_segment, smallest, biggest>).

    generate_on_device / free_on_device mirror gallatin.cuh:324 and :643.
    """

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def generate_on_device(cls, max_bytes, seed, print_info=False, boot=True, **cfg):
        config = default_config(**cfg)
        h = C.c_void_p()
        fn = lib().gal_create if boot else lib().gal_create_unbooted
        _check(fn(max_bytes, seed, C.byref(config), C.byref(h)), "gal_create")
        g = cls(h.value)
        if print_info:
            st = g.stats()
            print(f"Booted Gallatin with {st.num_trees} trees in range {config.min_size}-"
                  f"{config.max_size} and {max_bytes / 2**30:f} GB of memory {st.num_segments} segments")
        return g

    @staticmethod
    def free_on_device(g: "Gallatin"):
        g.close()

    def close(self):
        if self._h and self._h.value:
            _check(lib().gal_destroy(self._h), "gal_destroy")
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def device_state(self) -> int:
        return lib().gal_device_state(self._h)

    @property
    def arena_base(self) -> int:
        return lib().gal_arena_base(self._h)

    @property
    def arena_bytes(self) -> int:
        return lib().gal_arena_bytes(self._h)

    def stats(self) -> GalStats:
        s = GalStats()
        _check(lib().gal_get_stats(self._h, C.byref(s)), "gal_get_stats")
        return s

    def print_info(self):
        _check(lib().gal_print_stats(self._h), "gal_print_stats")

    def error_word(self) -> int:
        v = C.c_uint32()
        _check(lib().gal_last_error(self._h, C.byref(v)), "gal_last_error")
        return v.value

    def clear_error(self):
        _check(lib().gal_clear_error(self._h), "gal_clear_error")

    def error_info(self):
        """(site, a, b, recorded) of the first device error."""
        v = np.zeros(4, dtype=np.uint64)
        _check(lib().gal_error_info(self._h, v.ctypes.data), "gal_error_info")
        return tuple(int(x) for x in v)

    def dims(self) -> GalStateDims:
        d = GalStateDims()
        _check(lib().gal_state_dims_get(self._h, C.byref(d)), "gal_state_dims_get")
        return d

    def export(self) -> StateView:
        sv = StateView(self.dims())
        v = sv.cview()
        _check(lib().gal_export_state(self._h, C.byref(v)), "gal_export_state")
        sv.pull(v)
        return sv

    def export_noalloc(self) -> StateView:
        """export() without any device allocation (gal_export_state_noalloc)."""
        sv = StateView(self.dims())
        v = sv.cview()
        _check(lib().gal_export_state_noalloc(self._h, C.byref(v)), "gal_export_state_noalloc")
        sv.pull(v)
        return sv

    def load(self, sv: StateView):
        v = sv.cview()
        _check(lib().gal_import_state(self._h, C.byref(v)), "gal_import_state")

    def set_smid_override(self, smid: int):
        _check(lib().gal_set_smid_override(self._h, smid), "gal_set_smid_override")

    def set_policy(self, policy: int):
        _check(lib().gal_set_policy(self._h, policy), "gal_set_policy")

    # ---- device work (tensors or raw device pointers) ----
    def replay(self, ops: np.ndarray):
        """Serial replay by one device thread; returns (offsets, smid)."""
        import torch
        d_ops = torch.from_numpy(np.ascontiguousarray(ops, dtype=np.uint64).view(np.int64)).cuda()
        d_out = torch.empty_like(d_ops)
        d_smid = torch.zeros(1, dtype=torch.int32, device="cuda")
        _check(lib().gal_replay_trace(self._h, d_ops.data_ptr(), len(ops), d_out.data_ptr(),
                                      d_smid.data_ptr(), None), "gal_replay_trace")
        torch.cuda.synchronize()
        return d_out.cpu().numpy().view(np.uint64), int(d_smid.item())

    def replay_warp(self, steps: np.ndarray):
        """Warp-wide calls replayed by one warp (33 words per step); returns
        (32 offsets per step, smid)."""
        import torch
        steps = np.ascontiguousarray(steps, dtype=np.uint64)
        n = len(steps) // 33
        d_steps = torch.from_numpy(steps.view(np.int64)).cuda()
        d_out = torch.full((n * 32,), -1, dtype=torch.int64, device="cuda")
        d_smid = torch.zeros(1, dtype=torch.int32, device="cuda")
        _check(lib().gal_replay_warp_trace(self._h, d_steps.data_ptr(), n, d_out.data_ptr(),
                                           d_smid.data_ptr(), None), "gal_replay_warp_trace")
        torch.cuda.synchronize()
        return d_out.cpu().numpy().view(np.uint64), int(d_smid.item())

    def malloc_per_thread(self, sizes, out, stream=None):
        _check(lib().gal_malloc_per_thread(self._h, _ptr(sizes), sizes.numel(), _ptr(out), stream),
               "gal_malloc_per_thread")

    def free_per_thread(self, ptrs, stream=None):
        _check(lib().gal_free_per_thread(self._h, _ptr(ptrs), ptrs.numel(), stream), "gal_free_per_thread")

    def malloc_batched(self, sizes, out, stream=None):
        _check(lib().gal_malloc_batched(self._h, _ptr(sizes), sizes.numel(), _ptr(out), stream),
               "gal_malloc_batched")

    def free_batched(self, ptrs, stream=None):
        _check(lib().gal_free_batched(self._h, _ptr(ptrs), ptrs.numel(), stream), "gal_free_batched")

    def trim(self, stream=None):
        """Retire the pinned blocks and boot the slots again (quiescent only)."""
        _check(lib().gal_trim(self._h, stream), "gal_trim")

    def free_batched_n(self, ptrs, d_count, stream=None):
        """Free the first d_count[0] entries of ptrs (a one-element uint64/int64
        device tensor written by earlier work on the stream)."""
        _check(lib().gal_free_batched_n(self._h, _ptr(ptrs), _ptr(d_count), ptrs.numel(), stream),
               "gal_free_batched_n")

    def bench_churn(self, threads_per_round, rounds, seed, batched, use_graph, warmup, steps):
        """batched: True/False, or a mask (1: CTA-aggregated malloc, 2: CTA-aggregated free)."""
        ms = np.zeros(max(steps, 1), dtype=np.float32)
        r = ChurnResult()
        mode = (3 if batched else 0) if isinstance(batched, bool) else int(batched)
        _check(lib().gal_bench_churn(self._h, threads_per_round, rounds, seed, mode,
                                     int(use_graph), warmup, steps, ms.ctypes.data, C.byref(r)),
               "gal_bench_churn")
        return ms[:steps], r

    def bench_churn_e2e(self, host_sizes, threads_per_round, rounds, seed, warmup, steps, use_graph=False):
        ms = np.zeros(max(steps, 1), dtype=np.float32)
        r = ChurnResult()
        _check(lib().gal_bench_churn_e2e(self._h, _ptr(host_sizes), threads_per_round, rounds, seed,
                                         warmup, steps, ms.ctypes.data, C.byref(r), int(use_graph)),
               "gal_bench_churn_e2e")
        return ms[:steps], r

    def bench_latency(self, n, seed, batched):
        """(malloc_cycles, free_cycles) per request of one churn round."""
        m = np.zeros(n, dtype=np.uint32)
        f = np.zeros(n, dtype=np.uint32)
        _check(lib().gal_bench_latency(self._h, n, seed, int(batched), m.ctypes.data, f.ctypes.data),
               "gal_bench_latency")
        return m, f

    def bench_tables(self, offsets, seed, batched, dump_table=None, dump_cap=0):
        """The chained-hash-table workload (gal_tables.cu); offsets: uint64 prefix
        sums of the table sizes.  Returns (TablesResult, dumped keys, values)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        r = TablesResult()
        keys = np.zeros(max(dump_cap, 1), dtype=np.uint64)
        vals = np.zeros(max(dump_cap, 1), dtype=np.uint64)
        n = np.zeros(1, dtype=np.uint64)
        dump = dump_table is not None and dump_cap > 0
        _check(lib().gal_bench_tables(self._h, len(offsets) - 1, offsets.ctypes.data, seed, int(batched),
                                      C.byref(r), dump_table or 0,
                                      keys.ctypes.data if dump else None,
                                      vals.ctypes.data if dump else None, dump_cap,
                                      n.ctypes.data if dump else None), "gal_bench_tables")
        got = int(min(n[0], dump_cap)) if dump else 0
        return r, keys[:got], vals[:got]

    def bench_server(self, streams, server_pct=25, direct=False, use_graph=True, warmup=1, steps=3,
                     deadline_ms=5000):
        """The resident-server workload (gal_server.cu): streams are
        (requests, lo, hi, log_uniform, keep) tuples.  Returns (step ms, ServerResult)."""
        arr = (ServerStream * len(streams))(*[ServerStream(*x) for x in streams])
        ms = np.zeros(max(steps, 1), dtype=np.float32)
        r = ServerResult()
        _check(lib().gal_bench_server(self._h, arr, len(streams), server_pct, int(direct), int(use_graph),
                                      warmup, steps, deadline_ms, ms.ctypes.data, C.byref(r)),
               "gal_bench_server")
        return ms[:steps], r

    def bench_stamp(self, n, size, rounds=1):
        ms = np.zeros(2, dtype=np.float32)
        st = np.zeros(4, dtype=np.uint64)
        _check(lib().gal_bench_stamp(self._h, n, size, rounds, ms.ctypes.data, st.ctypes.data),
               "gal_bench_stamp")
        return ms, st


def churn_sizes(base_slot, n, seed):
    out = np.zeros(n, dtype=np.uint64)
    _check(lib().gal_churn_sizes(base_slot, n, seed, out.ctypes.data), "gal_churn_sizes")
    return out


def sector_probe(hot, per_sector):
    """Atomics/s on `hot` 8-byte counters packed per_sector to a 32-byte sector."""
    a = C.c_double()
    _check(lib().gal_bench_sector_probe(hot, per_sector, C.byref(a)), "gal_bench_sector_probe")
    return a.value


def atomic_peak():
    """(distinct-address, same-address) L2 atomicAdd.u32 rates in atomics/s."""
    a, b = C.c_double(), C.c_double()
    _check(lib().gal_bench_atomic_peak(C.byref(a), C.byref(b)), "gal_bench_atomic_peak")
    return a.value, b.value


# ---- process-global instance (global_allocator.cuh:41-97) ----
def init_global_allocator(num_bytes, seed, print_info=True, running_calloc=False, **cfg):
    if running_calloc:
        cfg["zero_fill"] = 1  # calloc mode: every allocation handed out zeroed
    config = default_config(**cfg)
    _check(lib().gal_init(num_bytes, seed, C.byref(config)), "gal_init")
    if print_info:
        global_allocator().print_info()


def free_global_allocator():
    _check(lib().gal_teardown(), "gal_teardown")


def global_allocator() -> Gallatin:
    h = lib().gal_global()
    if not h:
        raise GalError("global allocator not initialised")
    return Gallatin(h)


def print_global_stats():
    global_allocator().print_info()


__all__ = [
    "FAIL", "FREE_BIT", "GAL_POLICY_LOWEST", "GAL_POLICY_REFERENCE", "Gallatin", "GalError",
    "StateView", "atomic_peak", "churn_sizes", "sector_probe", "default_config", "free_global_allocator",
    "global_allocator", "init_global_allocator", "lib", "print_global_stats",
]
