"""CPU-side checks of the C ABI library (no GPU needed, no device calls).

The library loads, exports every entry point include/gallatin_gb300.h
declares, and rejects invalid configurations before touching a device.
"""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gallatin_gb300.h")


@pytest.fixture(scope="module")
def L():
    import gallatin_gb300
    from gallatin_gb300 import build
    if not os.path.exists(gallatin_gb300.LIB_PATH):
        build.build()
    return gallatin_gb300.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gal_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ["gal_create", "gal_destroy", "gal_init", "gal_teardown", "gal_get_stats",
                 "gal_last_error", "gal_device_state", "gal_export_state", "gal_import_state",
                 "gal_replay_trace", "gal_replay_warp_trace", "gal_malloc_per_thread", "gal_free_per_thread",
                 "gal_malloc_batched", "gal_free_batched"]:
        assert must in names


def test_library_exports_every_declared_symbol(L):
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert missing == []


def test_default_config_is_reference_geometry(L):
    import gallatin_gb300 as G
    cfg = G.default_config()
    assert (cfg.bytes_per_segment, cfg.min_size, cfg.max_size) == (16 << 20, 16, 4096)
    assert (cfg.pinned_slots_first, cfg.pinned_slots_min) == (128, 4)
    assert cfg.smid_override == -1 and cfg.subtree_policy == G.GAL_POLICY_REFERENCE
    assert cfg.team_width == 32
    assert (cfg.arena_kind, cfg.spare_blocks, cfg.zero_fill) == (G._abi.GAL_ARENA_DEVICE, 0, 0)


@pytest.mark.parametrize("ctype,mirror", [("gal_config", "GalConfig"), ("gal_stats", "GalStats"),
                                           ("gal_state_dims", "GalStateDims"),
                                           ("gal_state_view", "GalStateViewC")])
def test_ctypes_mirrors_have_the_header_layout(tmp_path, ctype, mirror):
    """Each ctypes mirror of a struct in include/gallatin_gb300.h has the C
    struct's size and field offsets (a C program compiled against the header
    prints them)."""
    import shutil
    import subprocess

    import gallatin_gb300 as G
    if not shutil.which("gcc"):
        pytest.skip("gcc absent")
    cls = getattr(G._abi, mirror)
    fields = [f[0] for f in cls._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"gallatin_gb300.h\"\n"
                   "int main(void) {\n" + f'  printf("%zu\\n", sizeof({ctype}));\n' +
                   "".join(f'  printf("%zu\\n", offsetof({ctype}, {f}));\n' for f in fields) +
                   "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got[0] == C.sizeof(cls)
    assert got[1:] == [getattr(cls, f).offset for f in fields]


@pytest.mark.parametrize("kw", [
    dict(bytes_per_segment=24 << 20),          # not a power of two
    dict(min_size=24),
    dict(max_size=8192),                       # segment < max * 4096 (gallatin.cuh:300)
    dict(max_size=8),                          # max < min
    dict(subtree_policy=7),
    dict(team_width=12),                       # not a power of two
    dict(team_width=64),                       # wider than a warp
    dict(arena_kind=3),                        # device, host or managed only
    dict(spare_blocks=2),                      # off or on
    dict(zero_fill=2),                         # off or on
    dict(block_layout=2),                      # dense or record
    dict(l2_fetch_bytes=48),                   # 0, 32, 64 or 128
    dict(gather_ahead=2),                      # off or on
])
def test_invalid_config_rejected_before_device_use(L, kw):
    import gallatin_gb300 as G
    cfg = G.default_config(**kw)
    h = C.c_void_p()
    assert L.gal_create(2 << 30, 42, C.byref(cfg), C.byref(h)) == G._abi.GAL_ERR_ARGS
    assert not h.value


def test_arena_smaller_than_a_segment_rejected(L):
    import gallatin_gb300 as G
    h = C.c_void_p()
    assert L.gal_create(1 << 20, 42, None, C.byref(h)) == G._abi.GAL_ERR_ARGS


def test_null_arguments_rejected(L):
    import gallatin_gb300 as G
    assert L.gal_destroy(None) == G._abi.GAL_ERR_ARGS
    assert L.gal_get_stats(None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_replay_trace(None, None, 0, None, None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_replay_warp_trace(None, None, 0, None, None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_export_state_noalloc(None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_job_launch(None, 0, 0, 0, None, None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_bench_server(None, None, 0, 0, 0, 0, 0, 0, 0, None, None) == G._abi.GAL_ERR_ARGS
    assert L.gal_global() is None


def test_job_grid_rule_matches_the_host_mirror(L):
    """gal_job_ctas and the served loop's admission estimate agree."""
    from gallatin_gb300.serve import job_ctas
    for kind in (0, 1):
        for n in (1, 1000, 1 << 18, 3 << 18, 1 << 20, 5 << 20, 1 << 24, 1 << 30):
            assert L.gal_job_ctas(kind, n) == job_ctas(kind, n)
