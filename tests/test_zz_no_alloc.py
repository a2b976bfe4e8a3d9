"""The allocation-free entry point segsort_pairs_u32_noalloc.

It exists for callers that cannot allocate device memory where they sort
(a framework's caching allocator that owns the device, real-time loops that
must not block in or fail on an allocation); its temporary storage is a fixed
scratch array inside the library.  These tests call it through the C ABI and
compare its output, bit for bit, with the allocating segsort_pairs_u32 on two
calls in a row, so the second call also shows that what the first left in the
shared scratch does not leak into the result.  The file sorts last so that a
run stopping at its first failure has already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest


def _sort_u32(torch, fn, keys, vals, off):
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    do = torch.from_numpy(off).cuda()
    rc = fn(dk.data_ptr(), dv.data_ptr(), len(keys), do.data_ptr(), len(off) - 1,
            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_no_alloc_matches_allocating_entry_point_on_two_calls(pkg, cuda, inst):
    L = pkg.lib()
    max_n = pkg.SEGSORT_NOALLOC_MAX_N
    # Both instances hold segments longer than the tile capacity, so the
    # long-segment path runs on the scratch array.
    cases = [
        (inst.lognormal_offsets(max_n, seed=31, empty_frac=0.02),
         inst.uniform_keys(max_n, seed=31, bits=32)),
        (inst.diff_offsets(300_000, 7, seed=32), inst.uniform_keys(300_000, seed=32, bits=6)),
    ]
    for off, keys in cases:
        assert np.diff(off).max() > 4096
        vals = np.arange(len(keys), dtype=np.uint32)
        rc_ref, k_ref, v_ref = _sort_u32(cuda, L.segsort_pairs_u32, keys, vals, off)
        rc, k, v = _sort_u32(cuda, L.segsort_pairs_u32_noalloc, keys, vals, off)
        assert rc_ref == pkg.SEGSORT_OK and rc == pkg.SEGSORT_OK
        assert pkg.device_status() == pkg.SEGSORT_OK
        assert np.array_equal(k, k_ref)
        assert np.array_equal(v, v_ref)


_FRESH_PROCESS = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, {root!r})
import __graft_entry__ as entry
pkg = entry.load_package()
inst = __import__(entry.PKG_NAME + ".instances", fromlist=["x"])
L = pkg.lib()
made, used = ctypes.c_int(), ctypes.c_uint64()
def pool():
    assert L.segsort_pool_bytes(ctypes.byref(made), ctypes.byref(used)) == 0
    return made.value, used.value
n = 300000
off = torch.from_numpy(inst.diff_offsets(n, 9, seed=91)).cuda()
k = torch.from_numpy(inst.uniform_keys(n, seed=91).view(np.int32)).cuda()
v = torch.arange(n, dtype=torch.int32, device="cuda")
st = torch.cuda.current_stream().cuda_stream
assert pool() == (0, 0)
for _ in range(2):
    assert L.segsort_pairs_u32_noalloc(k.data_ptr(), v.data_ptr(), n, off.data_ptr(), 9, st) == 0
    torch.cuda.synchronize()
    assert pool() == (0, 0), pool()
# the allocating entry point creates the pool on its first long-segment call
assert L.segsort_pairs_u32(k.data_ptr(), v.data_ptr(), n, off.data_ptr(), 9, st) == 0
torch.cuda.synchronize()
assert pool()[0] == 1, pool()
print("pool untouched by the allocation-free calls")
"""


@pytest.mark.gpu
def test_no_alloc_never_creates_the_library_pool(pkg, cuda):
    """In a fresh process, calls of the allocation-free entry point leave the
    library's own memory pool uncreated; the allocating entry point then
    creates it.  A regression that let the no-allocation path fall back to
    the pool would fail here even though its results stay exact."""
    import subprocess
    import sys
    from conftest import ROOT
    r = subprocess.run([sys.executable, "-c", _FRESH_PROCESS.format(root=str(ROOT))],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "pool untouched" in r.stdout


@pytest.mark.gpu
def test_no_alloc_rejects_sizes_beyond_its_scratch(pkg, cuda):
    L = pkg.lib()
    d = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    rc = L.segsort_pairs_u32_noalloc(d.data_ptr(), d.data_ptr(), pkg.SEGSORT_NOALLOC_MAX_N + 1,
                                     d.data_ptr(), 1, cuda.cuda.current_stream().cuda_stream)
    assert rc == pkg.SEGSORT_ERR_TOO_LARGE
