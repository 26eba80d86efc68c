"""Python side of the reference harness (TEST INFRASTRUCTURE ONLY).

Runs the reference allocator's own device code (oracle/_ref/ref_harness.cubin,
compiled from the reference sources by oracle/Makefile) through
oracle/_ref/libref_loader.so.  Needs a GPU; used by tests/golden/make_ref_golden.py
and by `bench.py --impl reference`.  Run it in its own process: it drives the
device through the driver API, not through torch.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from gallatin_gb300._abi import FAIL, GalStateDims, StateView

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# the reference built as Gallatin<seg, 16, 4096>, one cubin per segment size
CUBINS = {16: os.path.join(REF_DIR, "ref_harness.cubin"),
          64: os.path.join(REF_DIR, "ref_harness_64m.cubin")}
CUBIN = CUBINS[16]
LOADER = os.path.join(REF_DIR, "libref_loader.so")

_lib = None
_mods = {}


def available(segment_mib=16):
    return os.path.exists(CUBINS[segment_mib])


def _build_loader():
    src = os.path.join(HERE, "ref_loader.c")
    if not os.path.exists(LOADER) or os.path.getmtime(LOADER) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "_ref/libref_loader.so"])


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError(f"{CUBIN} missing: build it where the reference sources are "
                                    "(make -C oracle _ref/ref_harness.cubin)")
        _build_loader()
        L = C.CDLL(LOADER)
        L.ref_open.argtypes = [C.c_char_p]
        L.ref_module_geometry.argtypes = [C.c_int, C.c_void_p]
        L.ref_create.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]
        L.ref_malloc_sizes.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
        L.ref_free_ptrs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        L.ref_destroy.argtypes = [C.c_void_p]
        L.ref_replay.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
        L.ref_replay_warp.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
        L.ref_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_churn.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int, C.c_int,
                                C.c_void_p, C.c_void_p]
        L.ref_stamp.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p]
        L.ref_arena_base.restype = C.c_uint64
        L.ref_arena_base.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def module(segment_mib=16):
    """Module id of the cubin built for segment_mib MiB segments (loaded once)."""
    if segment_mib not in _mods:
        if not available(segment_mib):
            raise FileNotFoundError(f"{CUBINS[segment_mib]} missing")
        r = lib().ref_open(CUBINS[segment_mib].encode())
        if r < 0:
            raise RuntimeError(f"ref_open failed ({r})")
        _mods[segment_mib] = r
    return _mods[segment_mib]


BOOT_NONE, BOOT_ONE_THREAD, BOOT_RACY = 0, 1, 2


class RefGPU:
    """One instance of the reference's Gallatin<segment_mib MiB, 16, 4096> on the GPU."""

    def __init__(self, num_bytes, seed, boot=BOOT_ONE_THREAD, segment_mib=16):
        h = C.c_void_p()
        r = lib().ref_create(module(segment_mib), num_bytes, seed, boot, C.byref(h))
        if r != 0:
            raise RuntimeError(f"ref_create failed ({r})")
        self._h = h
        self.num_bytes = num_bytes
        self.segment_bytes = segment_mib << 20

    @property
    def arena_base(self):
        return int(lib().ref_arena_base(self._h))

    def malloc_sizes(self, sizes):
        """One device thread per request (host array in); returns (pointers, kernel ms)."""
        sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        out = np.zeros(len(sizes), dtype=np.uint64)
        ms = C.c_float()
        r = lib().ref_malloc_sizes(self._h, sizes.ctypes.data, len(sizes), out.ctypes.data, C.byref(ms))
        if r != 0:
            raise RuntimeError(f"ref_malloc_sizes failed ({r})")
        return out, ms.value

    def free_ptrs(self, ptrs):
        """One device thread per pointer (0 skipped); returns the kernel ms."""
        ptrs = np.ascontiguousarray(ptrs, dtype=np.uint64)
        ms = C.c_float()
        r = lib().ref_free_ptrs(self._h, ptrs.ctypes.data, len(ptrs), C.byref(ms))
        if r != 0:
            raise RuntimeError(f"ref_free_ptrs failed ({r})")
        return ms.value

    def close(self):
        if self._h:
            lib().ref_destroy(self._h)
            self._h = None

    def replay(self, ops):
        ops = np.ascontiguousarray(ops, dtype=np.uint64)
        out = np.full(len(ops), FAIL, dtype=np.uint64)
        smid = np.zeros(1, dtype=np.uint32)
        r = lib().ref_replay(self._h, ops.ctypes.data, len(ops), out.ctypes.data, smid.ctypes.data)
        if r != 0:
            raise RuntimeError(f"ref_replay failed ({r})")
        return out, int(smid[0])

    def replay_warp(self, steps):
        """Warp trace (33 words per step) by one warp; returns (offsets, smid)."""
        steps = np.ascontiguousarray(steps, dtype=np.uint64)
        n = len(steps) // 33
        out = np.full(n * 32, FAIL, dtype=np.uint64)
        smid = np.zeros(1, dtype=np.uint32)
        r = lib().ref_replay_warp(self._h, steps.ctypes.data, n, out.ctypes.data, smid.ctypes.data)
        if r != 0:
            raise RuntimeError(f"ref_replay_warp failed ({r})")
        return out, int(smid[0])

    def export(self, dims: GalStateDims):
        sv = StateView(dims)
        v = sv.cview()
        r = lib().ref_export(self._h, C.byref(dims), C.byref(v))
        if r != 0:
            raise RuntimeError(f"ref_export failed ({r})")
        sv.pull(v)
        return sv

    def churn(self, threads_per_round, rounds, seed, warmup, steps):
        ms = np.zeros(max(steps, 1), dtype=np.float32)
        st = np.zeros(4, dtype=np.uint64)
        r = lib().ref_churn(self._h, threads_per_round, rounds, seed, warmup, steps,
                            ms.ctypes.data, st.ctypes.data)
        if r != 0:
            raise RuntimeError(f"ref_churn failed ({r})")
        return ms[:steps], st

    def stamp(self, n, size, rounds=1):
        ms = np.zeros(2, dtype=np.float32)
        st = np.zeros(4, dtype=np.uint64)
        r = lib().ref_stamp(self._h, n, size, rounds, ms.ctypes.data, st.ctypes.data)
        if r != 0:
            raise RuntimeError(f"ref_stamp failed ({r})")
        return ms, st

