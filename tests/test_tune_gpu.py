"""GPU: the plain-call autotuner sorts its problem exactly, records a route
for the problem's class, and later plain calls of that class -- in this
process, or after the cache file is loaded -- take the route and stay exact.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from test_parity_gpu import check_both

pytestmark = pytest.mark.gpu


def test_tuner_sorts_records_and_routes(pkg, cuda, oracle, inst, tmp_path):
    torch = cuda
    L = pkg.lib()
    L.segsort_tune_clear()
    n = 1 << 20
    off = inst.lognormal_offsets(n, seed=95, empty_frac=0.02)
    keys = inst.uniform_keys(n, seed=95)
    vals = np.arange(n, dtype=np.uint32)
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    do = torch.from_numpy(off).cuda()
    cache = tmp_path / "routes.txt"
    r, st, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    rc = L.segsort_tune_pairs_u32(dk.data_ptr(), dv.data_ptr(), n, do.data_ptr(), len(off) - 1,
                                  torch.cuda.current_stream().cuda_stream, str(cache).encode(),
                                  ctypes.byref(r), ctypes.byref(st), ctypes.byref(c))
    assert rc == pkg.SEGSORT_OK
    torch.cuda.synchronize()
    assert pkg.device_status() == pkg.SEGSORT_OK
    ek, ev = oracle.segsort_numpy(keys, off, vals)
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), ek)
    assert np.array_equal(dv.cpu().numpy().view(np.uint32), ev)
    assert r.value in (4096, 1 << 15, 1 << 17, 1 << 30, pkg.get_param(pkg.PARAM_RADIX_MIN_32))
    assert c.value in (0, 1, 2)
    assert cache.read_text().startswith("plain k4 n20 len")
    # recorded for this process ...
    assert L.segsort_tune_lookup(4, n, len(off) - 1, None, None, None) == 1
    check_both(pkg, cuda, oracle, keys, off)
    # ... and loadable into a fresh table
    L.segsort_tune_clear()
    assert L.segsort_tune_load(str(cache).encode()) == 1
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=96, bits=5), off)
    L.segsort_tune_clear()
