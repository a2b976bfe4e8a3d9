"""CPU: the C-ABI library builds for sm_103a, loads, and exports every entry
point include/segsort.h declares.  Only host-side paths run here (argument
checks that return before any CUDA call, sizes, strings); no kernel runs."""
from __future__ import annotations

import ctypes
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "segsort.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(segsort_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("segsort_keys_u32", "segsort_pairs_u32", "segsort_pairs_u32_heads",
                 "segsort_workspace_bytes", "segsort_device_status"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    out = subprocess.run(["nm", "-D", "--defined-only", str(pkg.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (segsort_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_python_binding_covers_the_header(pkg):
    assert set(declared_functions()) == set(pkg.SIGNATURES)
    L = pkg.lib()
    for name in pkg.SIGNATURES:
        assert callable(getattr(L, name))


def test_library_is_built_for_sm_103a(pkg):
    from importlib import util
    spec = util.spec_from_file_location("_segsort_build_check", ROOT / "segmented-sorting_gb300" / "build.py")
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert all("sm_103a" in " ".join(mod._obj_cmd(u)) for u in mod.LIB_UNITS)


def test_run_time_parameters(pkg):
    """segsort_set_param / segsort_get_param are host-side only."""
    L = pkg.lib()
    saved = {p: pkg.get_param(p) for p in (pkg.PARAM_RADIX_MIN_32, pkg.PARAM_RADIX_MIN_64,
                                            pkg.PARAM_STREAM_MAX_AVG, pkg.PARAM_BUCKET_MIN_AVG,
                                            pkg.PARAM_MSD, pkg.PARAM_TINY_MAX_AVG)}
    assert saved[pkg.PARAM_RADIX_MIN_32] >= 4096 and saved[pkg.PARAM_RADIX_MIN_64] >= 4096
    assert saved[pkg.PARAM_BUCKET_MIN_AVG] == 128
    assert saved[pkg.PARAM_MSD] == 1 and saved[pkg.PARAM_TINY_MAX_AVG] == 8
    with pkg.params({pkg.PARAM_RADIX_MIN_32: 1 << 20, pkg.PARAM_STREAM_MAX_AVG: 0,
                     pkg.PARAM_BUCKET_MIN_AVG: 0, pkg.PARAM_MSD: 0, pkg.PARAM_TINY_MAX_AVG: 0}):
        assert pkg.get_param(pkg.PARAM_RADIX_MIN_32) == 1 << 20
        assert pkg.get_param(pkg.PARAM_STREAM_MAX_AVG) == 0
        assert pkg.get_param(pkg.PARAM_BUCKET_MIN_AVG) == 0
        assert pkg.get_param(pkg.PARAM_MSD) == 0
        assert pkg.get_param(pkg.PARAM_TINY_MAX_AVG) == 0
    assert {p: pkg.get_param(p) for p in saved} == saved
    assert L.segsort_set_param(pkg.PARAM_BUCKET_MIN_AVG, -5) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_set_param(pkg.PARAM_MSD, 2) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_set_param(pkg.PARAM_TINY_MAX_AVG, -1) == pkg.SEGSORT_ERR_INVALID_ARG
    # below the floor, negative, unknown parameter, missing output
    assert L.segsort_set_param(pkg.PARAM_RADIX_MIN_32, 4095) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_set_param(pkg.PARAM_RADIX_MIN_64, 100) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_set_param(pkg.PARAM_STREAM_MAX_AVG, -1) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_set_param(99, 1) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_get_param(99, ctypes.byref(ctypes.c_int64())) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_get_param(pkg.PARAM_RADIX_MIN_32, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert {p: pkg.get_param(p) for p in saved} == saved


def test_host_side_argument_checks(pkg):
    L = pkg.lib()
    # n == 0 or nseg == 0: nothing to do, no device access
    assert L.segsort_keys_u32(None, 0, None, 0, None) == pkg.SEGSORT_OK
    assert L.segsort_pairs_u32(None, None, 0, None, 5, None) == pkg.SEGSORT_OK
    # negative sizes and null pointers are rejected before any CUDA call
    assert L.segsort_keys_u32(None, -1, None, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_keys_u32(None, 10, None, -1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_keys_u32(None, 10, None, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_pairs_f32(ctypes.c_void_p(16), None, 10, ctypes.c_void_p(16), 1,
                               None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_keys_u64(ctypes.c_void_p(16), 1 << 30, ctypes.c_void_p(16), 1,
                              None) == pkg.SEGSORT_ERR_TOO_LARGE
    # the explicit-workspace form refuses a missing workspace when one is needed
    assert L.segsort_pairs_u32_ws(ctypes.c_void_p(16), ctypes.c_void_p(16), 1 << 20,
                                  ctypes.c_void_p(16), 1, None, 0,
                                  None) == pkg.SEGSORT_ERR_WORKSPACE


def test_workspace_sizes(pkg):
    L = pkg.lib()
    # no segment can exceed the tile capacity: no workspace at all
    assert L.segsort_workspace_bytes(4096, 1, 4, 4) == 0
    assert L.segsort_workspace_bytes(2048, 1, 8, 4) == 0
    n = 1 << 24
    ws_pairs = L.segsort_workspace_bytes(n, 1, 4, 4)
    ws_keys = L.segsort_workspace_bytes(n, 1, 4, 0)
    # the ping-pong copy of the keys (and values) dominates
    assert ws_pairs >= 8 * n and ws_keys >= 4 * n and ws_pairs - ws_keys >= 4 * n
    assert ws_pairs < 11 * n
    assert L.segsort_workspace_bytes(n, 1, 8, 4) >= 12 * n


def test_error_strings_and_version(pkg):
    L = pkg.lib()
    for code in range(0, -7, -1):
        assert L.segsort_error_string(code)
    assert L.segsort_version() >= 100


def test_batch_host_side_argument_checks(pkg):
    """The batched entry points validate every item before any CUDA call."""
    L = pkg.lib()
    P = ctypes.c_void_p(16)

    def items(*specs):
        return (pkg.BatchItem * len(specs))(*[pkg.BatchItem(*s) for s in specs])

    ok = (0, 0, 16, 16, 100, 16, 1, 0)
    # nothing to sort: empty list, or only empty items
    assert L.segsort_pairs_batch(None, 0, None) == pkg.SEGSORT_OK
    assert L.segsort_pairs_batch(items((0, 0, None, None, 0, None, 0, 0)), 1, None) == pkg.SEGSORT_OK
    assert L.segsort_pairs_batch(None, 3, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_pairs_batch(items(ok), -1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    bad = [
        (7, 0, 16, 16, 100, 16, 1, 0),      # unknown key type
        (0, 2, 16, 16, 100, 16, 1, 0),      # heads flag not 0/1
        (0, 0, 16, 16, -1, 16, 1, 0),       # n < 0
        (0, 0, 16, 16, 100, 16, -1, 0),     # nseg < 0
        (0, 0, None, 16, 100, 16, 1, 0),    # null keys
        (2, 0, 16, None, 100, 16, 1, 0),    # null values
        (3, 0, 16, 16, 100, None, 1, 0),    # null offsets
    ]
    for b in bad:
        assert L.segsort_pairs_batch(items(ok, b), 2, None) == pkg.SEGSORT_ERR_INVALID_ARG, b
    assert L.segsort_pairs_batch(items((0, 0, 16, 16, 1 << 30, 16, 1, 0)), 1,
                                 None) == pkg.SEGSORT_ERR_TOO_LARGE
    # one key type's items together at most 2^31 - 1 elements
    big = (1, 0, 16, 16, (1 << 30) - 1, 16, 1, 0)
    assert L.segsort_pairs_batch(items(big, big, big), 3, None) == pkg.SEGSORT_ERR_TOO_LARGE
    plan = ctypes.c_void_p()
    assert L.segsort_batch_plan_create(items(bad[0]), 1, ctypes.byref(plan)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert not plan.value
    assert L.segsort_batch_plan_create(items(ok), 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_batch_plan_launch(None, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_batch_plan_workspace_bytes(None) == 0
    L.segsort_batch_plan_destroy(None)
    del P


def test_server_host_side_argument_checks(pkg):
    """Server entry points reject bad arguments before any CUDA call."""
    L = pkg.lib()
    h = ctypes.c_void_p()
    assert L.segsort_server_create(0, 0, 0, 0, ctypes.byref(h)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_create(1 << 30, -1, 0, 0, ctypes.byref(h)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_create(1 << 30, 0, -1, 0, ctypes.byref(h)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_create(1 << 30, 0, 0, 9, ctypes.byref(h)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_create(1 << 30, 0, 0, 0, None) == pkg.SEGSORT_ERR_INVALID_ARG
    t = ctypes.c_uint64()
    assert L.segsort_server_submit(None, None, None, 0, None, 0, None, None,
                                   ctypes.byref(t)) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_wait(None, 0, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_drain(None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_server_get_stats(None, None) == pkg.SEGSORT_ERR_INVALID_ARG
    L.segsort_server_destroy(None)
    # the batch workspace query is host arithmetic
    items = (pkg.BatchItem * 2)(pkg.BatchItem(0, 0, 16, 16, 1 << 20, 16, 4, 0),
                                pkg.BatchItem(3, 0, 16, 16, 5000, 16, 2, 0))
    ws = L.segsort_batch_workspace_bytes(items, 2)
    # at least the ping-pong copies of both items' keys and values
    assert ws > 8 * (1 << 20) + 12 * 5000
    assert L.segsort_batch_workspace_bytes(items, -1) == 0


def test_extension_host_side_argument_checks(pkg):
    """Descending, top-k and 64-bit-value entry points reject bad arguments
    before any CUDA call, and return at once when there is nothing to sort."""
    L = pkg.lib()
    P = ctypes.c_void_p(16)
    for t in pkg.KEY_TYPES:
        f = getattr(L, f"segsort_pairs_{t}_desc")
        assert f(None, None, 0, None, 0, None) == pkg.SEGSORT_OK
        assert f(None, None, -1, None, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
        assert f(P, None, 10, P, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
        assert f(P, P, 1 << 30, P, 1, None) == pkg.SEGSORT_ERR_TOO_LARGE
        g = getattr(L, f"segsort_pairs_{t}_v64")
        assert g(None, None, 0, None, 0, None) == pkg.SEGSORT_OK
        assert g(P, None, 10, P, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
        assert g(P, P, 1 << 30, P, 1, None) == pkg.SEGSORT_ERR_TOO_LARGE
    assert L.segsort_keys_u32_desc(None, 10, P, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert L.segsort_keys_f32_desc(P, 10, None, 1, None) == pkg.SEGSORT_ERR_INVALID_ARG
    for t in ("u32", "f32"):
        f = getattr(L, f"segsort_pairs_{t}_topk")
        assert f(P, P, 10, P, 1, 0, 0, P, P, None, None) == pkg.SEGSORT_OK   # k = 0
        assert f(P, P, 10, P, 1, -1, 0, P, P, None, None) == pkg.SEGSORT_ERR_INVALID_ARG
        assert f(P, P, 10, P, 1, 4, 0, None, P, None, None) == pkg.SEGSORT_ERR_INVALID_ARG
        assert f(P, None, 10, P, 1, 4, 0, P, P, None, None) == pkg.SEGSORT_ERR_INVALID_ARG


def test_reduce_by_key_host_side_argument_checks(pkg):
    L = pkg.lib()
    P = ctypes.c_void_p(16)
    f = L.segsort_pairs_u32_reduce_by_key
    assert f(None, None, 0, None, 0, None, None, None, None, None) == pkg.SEGSORT_OK
    assert f(P, P, -1, P, 1, P, P, P, P, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert f(P, P, 10, P, 1, P, P, P, None, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert f(P, None, 10, P, 1, P, P, P, P, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert f(P, P, 10, P, 1, P, None, P, P, None) == pkg.SEGSORT_ERR_INVALID_ARG
    assert f(P, P, 1 << 30, P, 1, P, P, P, P, None) == pkg.SEGSORT_ERR_TOO_LARGE


def test_batch_tune_rejects_a_missing_plan(pkg):
    L = pkg.lib()
    k = ctypes.c_int32()
    assert L.segsort_batch_plan_tune(None, None, None, ctypes.byref(k)) == pkg.SEGSORT_ERR_INVALID_ARG


def test_tuned_route_table(pkg, tmp_path):
    """segsort_tune_load / _lookup / _clear are host-only: the cache file's
    plain-call lines become the routes of their classes; other lines are
    skipped."""
    L = pkg.lib()
    cache = tmp_path / "routes.txt"
    cache.write_text("t1-n24-max20-len10 3\n"             # a batch-plan line
                     "plain k4 n24 len10 32768 32 2\n"
                     "plain k8 n20 len4 4096 0 0 64 0\n"  # with the bucket and MSD fields
                     "plain k4 n24 len10 131072 0 1\n"     # a later line wins
                     "plain k4 n22 len10 131072 0 1 128 2\n"  # MSD field out of range
                     "garbage\n")
    L.segsort_tune_clear()
    r, st, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    assert L.segsort_tune_lookup(4, 1 << 24, 1 << 14, ctypes.byref(r), ctypes.byref(st),
                                 ctypes.byref(c)) == 0
    assert L.segsort_tune_load(str(cache).encode()) == 3
    assert L.segsort_tune_lookup(4, 1 << 24, 1 << 14, ctypes.byref(r), ctypes.byref(st),
                                 ctypes.byref(c)) == 1
    assert (r.value, st.value, c.value) == (131072, 0, 1)
    # the class is log2 n and log2 (n / nseg): 2^24 + 5 keys in 2^14 segments share it
    assert L.segsort_tune_lookup(4, (1 << 24) + 5, 1 << 14, None, None, None) == 1
    assert L.segsort_tune_lookup(8, (1 << 20) + 100, 1 << 16, ctypes.byref(r), None, None) == 1
    assert r.value == 4096
    assert L.segsort_tune_lookup(4, 1 << 23, 1 << 14, None, None, None) == 0
    assert L.segsort_tune_load(str(tmp_path / "missing").encode()) == pkg.SEGSORT_ERR_INVALID_ARG
    L.segsort_tune_clear()
    assert L.segsort_tune_lookup(4, 1 << 24, 1 << 14, None, None, None) == 0
