"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the gallatin_gb300 package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from gallatin_gb300._abi import FAIL, GalStateDims, StateView, GAL_POLICY_REFERENCE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

FIX_GATHER_EXIT_ROLLBACK = 0x1
FIX_LEFTOVER_COMPLETES = 0x2
FIX_RUN_BELOW_ARENA = 0x4
FIX_RUN_RETURN_SUMMARY = 0x8
# the product fixes these reference defects; parity runs against the product use them
PRODUCT_FIXES = (FIX_GATHER_EXIT_ROLLBACK | FIX_LEFTOVER_COMPLETES | FIX_RUN_BELOW_ARENA
                 | FIX_RUN_RETURN_SUMMARY)

_lib = None


def build(force=False):
    """Compile liboracle.so with gcc (no GPU, no CUDA needed)."""
    src = os.path.join(HERE, "gal_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                 C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_boot_one_thread.argtypes = [C.c_void_p]
        L.orc_trim.argtypes = [C.c_void_p]
        L.orc_set_spares.argtypes = [C.c_void_p, C.c_int]
        L.orc_malloc.restype = C.c_uint64
        L.orc_malloc.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64]
        L.orc_free.argtypes = [C.c_void_p, C.c_uint64]
        L.orc_replay.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p]
        L.orc_replay_warp.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64,
                                      C.c_void_p]
        L.orc_dims.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_export.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_import.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_gen_serial_trace.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64,
                                           C.c_uint64, C.c_void_p]
        L.orc_gen_trace_log.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.c_void_p]
        L.orc_murmur64a_u64.restype = C.c_uint64
        L.orc_murmur64a_u64.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_arena_bytes.restype = C.c_uint64
        L.orc_arena_bytes.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def gen_serial_trace(seed=7, nops=4096, malloc_pct=60, quantum=16, steps=256):
    """The serial trace: splitmix64(seed); 60% malloc / 40% free of a random live op."""
    ops = np.zeros(nops, dtype=np.uint64)
    lib().orc_gen_serial_trace(seed, nops, malloc_pct, quantum, steps, ops.ctypes.data)
    return ops


def gen_log_trace(seed, nops, malloc_pct, lo_bits, hi_bits):
    """Log-uniform sizes between 2^lo_bits and 2^hi_bits (see gal_oracle.c)."""
    ops = np.zeros(nops, dtype=np.uint64)
    lib().orc_gen_trace_log(seed, nops, malloc_pct, lo_bits, hi_bits, ops.ctypes.data)
    return ops


def gen_leftover_trace(slice_size):
    """Fill one block of the largest size class but its last slice, free all
    of it, then ask for a run of two slices: the run does not fit, so the one
    slice left over is credited back (block.cuh:267-281) and completes the
    block's free count.  Then free the run."""
    n = 4095
    ops = [slice_size] * n + [(1 << 63) | i for i in range(n)] + [2 * slice_size]
    ops.append((1 << 63) | (len(ops) - 1))
    return np.array(ops, dtype=np.uint64)


WARP_MALLOC, WARP_FREE = 0, 1


def gen_warp_trace(seed, nsteps, malloc_pct=65, tree_weights=(6, 4, 3, 2, 1, 1, 1, 1, 2),
                   big_pct=30, drain=True, min_size=16):
    """A trace of warp-wide calls (33 words per step, see orc_replay_warp).

    Malloc steps: a lane mask (the full warp one time in three, else random
    bits) and one slice class for the whole step, drawn by tree_weights (one
    weight per class of min_size << t bytes); sizes uniform inside the class
    (the last class takes big-slice sizes of 2, 4 or 8 slices in big_pct
    percent of its lanes, mixed with single slices).  Free
    steps free up to 32 earlier results chosen at random.  With drain, steps
    freeing everything still live close the trace.  numpy PCG64 seeded with
    `seed`; the fixtures keep the generated steps themselves."""
    rng = np.random.default_rng(seed)
    w = np.asarray(tree_weights, dtype=np.float64)
    w /= w.sum()
    steps, live = [], []

    def free_step(targets):
        row = np.zeros(33, dtype=np.uint64)
        lanes = np.sort(rng.choice(32, size=len(targets), replace=False))
        mask = 0
        for lane, t in zip(lanes, targets):
            row[1 + lane] = t
            mask |= 1 << int(lane)
        row[0] = (WARP_FREE << 32) | mask
        steps.append(row)

    for _ in range(nsteps):
        i = len(steps)
        if live and rng.integers(100) >= malloc_pct:
            k = int(min(len(live), rng.integers(1, 33)))
            pick = rng.choice(len(live), size=k, replace=False)
            targets = [live[j] for j in pick]
            for j in sorted(pick, reverse=True):
                live[j] = live[-1]
                live.pop()
            free_step(targets)
            continue
        mask = 0xFFFFFFFF if rng.integers(3) == 0 else int(rng.integers(1, 1 << 32))
        t = int(rng.choice(len(w), p=w))
        row = np.zeros(33, dtype=np.uint64)
        for lane in range(32):
            if not (mask >> lane) & 1:
                continue
            top = min_size << t
            if t == len(w) - 1 and rng.integers(100) < big_pct:
                c = int(rng.choice([2, 4, 8]))
                size = int(rng.integers(top * c // 2 + 1, top * c + 1))
            else:
                lo = 1 if t == 0 else top // 2 + 1
                size = int(rng.integers(lo, top + 1))
            row[1 + lane] = size
            live.append(i * 32 + lane)
        row[0] = (WARP_MALLOC << 32) | mask
        steps.append(row)
    if drain:
        order = rng.permutation(len(live))
        for s0 in range(0, len(order), 32):
            free_step([live[j] for j in order[s0:s0 + 32]])
    return np.concatenate(steps) if steps else np.zeros(0, dtype=np.uint64)


def murmur64a(key, seed):
    return int(lib().orc_murmur64a_u64(key, seed))


class Oracle:
    """One allocator instance of the CPU model."""

    def __init__(self, num_bytes, seed, bytes_per_segment=16 << 20, min_size=16, max_size=4096,
                 pinned_first=128, pinned_min=4, fixes=PRODUCT_FIXES, policy=GAL_POLICY_REFERENCE,
                 boot=True, spares=False):
        self._h = lib().orc_create(num_bytes, seed, bytes_per_segment, min_size, max_size,
                                   pinned_first, pinned_min, fixes, policy)
        if not self._h:
            raise RuntimeError("orc_create failed")
        lib().orc_set_spares(self._h, 1 if spares else 0)
        self.bytes_per_segment = bytes_per_segment
        if boot:
            r = lib().orc_boot_one_thread(self._h)
            if r != 0:
                raise RuntimeError(f"oracle boot failed ({r})")

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def malloc(self, size, smid=0, tid=0):
        return int(lib().orc_malloc(self._h, size, smid, tid))

    def trim(self):
        """Retire every pinned block, then boot the slots again (gal_trim)."""
        r = lib().orc_trim(self._h)
        if r != 0:
            raise RuntimeError(f"oracle trim failed ({r})")

    def free(self, byte_offset):
        lib().orc_free(self._h, byte_offset)

    def replay(self, ops, smid=0, tid=0):
        ops = np.ascontiguousarray(ops, dtype=np.uint64)
        out = np.full(len(ops), FAIL, dtype=np.uint64)
        r = lib().orc_replay(self._h, ops.ctypes.data, len(ops), smid, tid, out.ctypes.data)
        if r != 0:
            raise ValueError("bad trace")
        return out

    def replay_warp(self, steps, smid=0, tid0=0):
        """Warp trace (33 words per step) by one modelled warp of thread ids
        tid0..tid0+31; returns 32 offsets per step."""
        steps = np.ascontiguousarray(steps, dtype=np.uint64)
        n = len(steps) // 33
        out = np.full(n * 32, FAIL, dtype=np.uint64)
        r = lib().orc_replay_warp(self._h, steps.ctypes.data, n, smid, tid0, out.ctypes.data)
        if r != 0:
            raise ValueError("bad warp trace")
        return out

    def dims(self):
        d = GalStateDims()
        lib().orc_dims(self._h, C.byref(d))
        return d

    def export(self):
        sv = StateView(self.dims())
        v = sv.cview()
        lib().orc_export(self._h, C.byref(v))
        sv.pull(v)
        return sv

    def load(self, sv: StateView):
        v = sv.cview()
        lib().orc_import(self._h, C.byref(v))

    @property
    def arena_bytes(self):
        return int(lib().orc_arena_bytes(self._h))
