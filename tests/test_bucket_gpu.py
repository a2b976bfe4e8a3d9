"""GPU parity of the bucket route of the tile sort, through the C ABI,
against the oracle.

Problems whose average segment is at least SEGSORT_PARAM_BUCKET_MIN_AVG keys
(and not short enough for the streamed kernel) are tile-sorted by the bucket
kernel: every chunk of whole segments is bucket-sorted by scaled key value,
and chunks it refuses (segments shorter than 128 keys on average, skewed or
low-entropy keys) are listed for the comparison sort.  Every case here runs
with the route forced on (threshold 1) and off (0), so the bucket sort, its
refusal path and the comparison sort all stay covered whatever the
defaults are.  Bar: bit-exact keys and values, stable order of equal keys
included.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_parity_gpu import check_both

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["bucket", "compare"])
def route(request, pkg, cuda):
    v = 1 if request.param == "bucket" else 0
    with pkg.params({pkg.PARAM_BUCKET_MIN_AVG: v, pkg.PARAM_STREAM_MAX_AVG: 0}):
        yield request.param


@pytest.mark.parametrize("length", [40, 128, 129, 300, 1000, 2048, 2049, 4095, 4096])
@pytest.mark.parametrize("bits", [32, 12, 4, 1])
def test_equal_segments(pkg, cuda, oracle, inst, route, length, bits):
    n = (1 << 17) // length * length + length // 2  # ragged last segment
    off = np.concatenate([inst.equal_offsets(n - length // 2, length), [n]]).astype(np.int32)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=length * 7 + bits, bits=bits), off)


def test_lognormal_and_zipf(pkg, cuda, oracle, inst, route):
    off = inst.lognormal_offsets(1 << 19, seed=91, empty_frac=0.02)
    check_both(pkg, cuda, oracle, inst.uniform_keys(1 << 19, seed=91), off)
    check_both(pkg, cuda, oracle, inst.zipf_keys(1 << 19, seed=92), off)


def test_sorted_reversed_and_equal_keys(pkg, cuda, oracle, inst, route):
    n, length = 1 << 17, 1000
    off = np.concatenate([inst.equal_offsets(n // length * length, length), [n]]).astype(np.int32)
    asc = np.arange(n, dtype=np.uint32) * np.uint32(40503)
    for keys in (np.sort(asc), np.sort(asc)[::-1].copy(), np.full(n, 7, np.uint32),
                 (np.arange(n) % 3).astype(np.uint32)):
        check_both(pkg, cuda, oracle, keys, off)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_key_types(pkg, cuda, oracle, inst, route, dtype):
    rng = np.random.default_rng(93)
    lens = rng.integers(100, 3000, 150)
    lens[::17] = 0
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 1e3).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-42, -1e-42], np.float32)
        keys[rng.integers(0, n, 500)] = specials[rng.integers(0, len(specials), 500)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=94).view(np.int32).copy()
        keys[::13] = np.int32(-2147483648)
        keys[::29] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=95, bits=64, dtype=np.uint64)
        keys[::5] &= np.uint64(0xFFFFFFFF)
    check_both(pkg, cuda, oracle, keys, off)


def test_runs_of_long_segments(pkg, cuda, oracle, inst, route):
    """Segments on the merge route: their CAP-runs are bucket-sorted into the
    buffer the first merge pass reads (the temporary one for an odd pass
    count)."""
    lens = [5000, 9000, 20000, 4097, 12289, 300, 64000]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    with pkg.params({pkg.PARAM_RADIX_MIN_32: 1 << 30}):
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=96), off)
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=97, bits=6), off)


def test_heads_only_offsets(pkg, cuda, oracle, inst, route):
    off = inst.diff_offsets(200000, 150, seed=98)
    check_both(pkg, cuda, oracle, inst.uniform_keys(200000, seed=98), off[:-1], heads=True)
