"""GPU parity of the two routes for segments longer than a tile, through the
C ABI, against the oracle.

Segments longer than the radix threshold (SEGSORT_PARAM_RADIX_MIN_32 / _64)
are sorted by LSD radix passes, shorter long segments by merge passes over
tile-sorted runs.  Every case here runs twice: with the threshold at its
floor (every long segment takes the radix passes) and above every length
(every long segment takes the merge passes), so both routes stay covered
whatever the defaults are.  Bar: bit-exact keys and values, stable order of
equal keys included.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_parity_gpu import assert_stable_sorted, check_both, gpu_sort, _u32_bits

pytestmark = pytest.mark.gpu

RADIX_FLOOR = 4096


@pytest.fixture(params=["radix", "merge"])
def route(request, pkg, cuda):
    v = RADIX_FLOOR if request.param == "radix" else 1 << 30
    with pkg.params({pkg.PARAM_RADIX_MIN_32: v, pkg.PARAM_RADIX_MIN_64: v}):
        yield request.param


@pytest.mark.parametrize("length", [4097, 5000, 8191, 8192, 8193, 12289, 65536, 100000, 300000])
def test_long_equal_segments(pkg, cuda, oracle, inst, route, length):
    n = max(length * 3, 1 << 18) // length * length + length // 3  # ragged tail segment
    off = np.concatenate([inst.equal_offsets(n - length // 3, length), [n]]).astype(np.int32)
    for bits in (32, 4):
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=length + bits, bits=bits), off)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_long_key_types(pkg, cuda, oracle, inst, route, dtype):
    rng = np.random.default_rng(50)
    lens = [3, 5000, 0, 9000, 4097, 70000, 1, 4096, 200000, 12]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 1e4).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 1e-42, -1e-42],
                            np.float32)
        keys[rng.integers(0, n, 3000)] = specials[rng.integers(0, len(specials), 3000)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=51).view(np.int32).copy()
        keys[::7] = np.int32(-2147483648)
        keys[::11] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=52, bits=64, dtype=np.uint64)
        keys[::3] &= np.uint64(0xFFFF)
        keys[::19] = np.uint64(0xFFFFFFFFFFFFFFFF)
    check_both(pkg, cuda, oracle, keys, off)


def test_long_random_cuts_and_lognormal(pkg, cuda, oracle, inst, route):
    for nseg, n, seed in [(1, 400000, 61), (9, 300000, 62), (40, 500000, 63)]:
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=seed), inst.diff_offsets(n, nseg, seed))
    off = inst.lognormal_offsets(1 << 20, seed=64, empty_frac=0.02)
    check_both(pkg, cuda, oracle, inst.zipf_keys(1 << 20, seed=64), off)


@pytest.mark.parametrize("shape", ["one_digit", "two_digits", "three_digits", "all_equal",
                                   "top_digit_only"])
def test_radix_digits_that_do_not_vary(pkg, cuda, oracle, inst, shape):
    """Keys whose digit positions are partly constant: the radix route skips
    those passes, ends in the temporary buffers after an odd number of
    passes and copies back.  Runs with every long segment on the radix
    route."""
    n = 300000
    x = inst.uniform_keys(n, seed=70, bits=32)
    keys = {"one_digit": x & 0xFF, "two_digits": (x & 0xFF) | ((x >> 8) & 0xFF) << 16,
            "three_digits": x & 0xFFFFFF, "all_equal": np.full(n, 0xABCD1234, np.uint32),
            "top_digit_only": (x & 0xFF) << 24}[shape].astype(np.uint32)
    off = inst.diff_offsets(n, 7, seed=71)
    with pkg.params({pkg.PARAM_RADIX_MIN_32: RADIX_FLOOR}):
        check_both(pkg, cuda, oracle, keys, off)
        u = keys.astype(np.uint64) | (keys.astype(np.uint64) << np.uint64(40))
        with pkg.params({pkg.PARAM_RADIX_MIN_64: RADIX_FLOOR}):
            check_both(pkg, cuda, oracle, u, off)


def test_radix_segments_among_merge_and_tile_segments(pkg, cuda, oracle, inst):
    """A threshold between the lengths sends some long segments to each
    route in the same call, beside short segments."""
    rng = np.random.default_rng(72)
    lens = np.concatenate([rng.integers(0, 40, 3000), [5000, 20000, 70000, 9000, 150000],
                           rng.integers(4000, 30000, 12)])
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    with pkg.params({pkg.PARAM_RADIX_MIN_32: 16384}):
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=73, bits=32), off)
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=74, bits=3), off)


def test_caller_workspace_serves_every_threshold(pkg, cuda, oracle, inst, route):
    n = 300000
    off = inst.diff_offsets(n, 5, seed=75)
    keys = inst.uniform_keys(n, seed=75)
    vals = np.arange(n, dtype=np.uint32)
    k, v = gpu_sort(pkg, cuda, keys, off, vals, ws=pkg.workspace_bytes(n, 5, 4, 4))
    ek, ev = oracle.segsort_numpy(keys, off, vals)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("log_len", [13, 16, 20])
def test_cfg2_long_lengths_both_routes(pkg, cuda, inst, route, log_len):
    torch = cuda
    n = 1 << 24
    off = inst.equal_offsets(n, 1 << log_len)
    for bits in (32, 4):
        keys = inst.uniform_keys(n, seed=log_len + 100, bits=bits)
        dk = torch.from_numpy(keys.view(np.int32)).cuda()
        before = _u32_bits(dk)
        dv = torch.arange(n, dtype=torch.int32, device="cuda")
        dof = torch.from_numpy(off).cuda()
        rc = pkg.lib().segsort_pairs_u32(dk.data_ptr(), dv.data_ptr(), n, dof.data_ptr(),
                                         len(off) - 1, torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert pkg.device_status() == 0
        assert_stable_sorted(torch, before, _u32_bits(dk), dv.long(), off)
