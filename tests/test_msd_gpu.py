"""GPU parity of the MSD route for radix segments, through the C ABI,
against the oracle.

A call whose average segment is longer than the radix threshold sorts each
radix segment whose keys vary in at least three 8-bit digits by one stable
radix pass on its top varying digit, then tile-sorts the 256 sub-buckets
(merge passes for a sub-bucket longer than a tile); the other radix segments
run all their LSD passes and are skipped by the second stage.  The radix
threshold is put at its floor (4096) so that small problems take the route;
every case runs with the route on and off.  Bar: bit-exact keys and values,
stable order of equal keys included.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_parity_gpu import check_both

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["msd", "lsd"])
def route(request, pkg, cuda):
    with pkg.params({pkg.PARAM_MSD: 1 if request.param == "msd" else 0,
                     pkg.PARAM_RADIX_MIN_32: 4096, pkg.PARAM_RADIX_MIN_64: 4096}):
        yield request.param


@pytest.mark.parametrize("length", [4097, 5000, 20000, 70000, 300000])
@pytest.mark.parametrize("bits", [32, 24, 20, 12, 4, 0])
def test_equal_segments(pkg, cuda, oracle, inst, route, length, bits):
    n = max(length * 3, 1 << 18) // length * length + length // 3  # ragged tail segment
    off = np.concatenate([inst.equal_offsets(n - length // 3, length), [n]]).astype(np.int32)
    keys = inst.uniform_keys(n, seed=length + bits, bits=max(bits, 1))
    if bits == 0:
        keys[:] = 0xA5A5A5A5
    check_both(pkg, cuda, oracle, keys, off)


def test_mixed_lengths_and_empty_segments(pkg, cuda, oracle, inst, route):
    """Radix segments among merge-route, tile and empty segments (an empty
    segment right before a radix segment shares its begin)."""
    rng = np.random.default_rng(101)
    lens = [0, 9000, 0, 0, 200000, 3, 40, 0, 70000, 4096, 4097, 0, 150000, 12, 0]
    lens += list(rng.integers(0, 2000, 40))
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=102), off)
    check_both(pkg, cuda, oracle, inst.zipf_keys(n, seed=103), off)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=104), off[:-1], heads=True)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_key_types(pkg, cuda, oracle, inst, route, dtype):
    rng = np.random.default_rng(105)
    lens = [30000, 5000, 120000, 0, 64000, 7]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 1e5).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-42, -1e-42], np.float32)
        keys[rng.integers(0, n, 2000)] = specials[rng.integers(0, len(specials), 2000)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=106).view(np.int32).copy()
        keys[::11] = np.int32(-2147483648)
        keys[::23] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=107, bits=64, dtype=np.uint64)
        keys[::9] >>= np.uint64(40)
    check_both(pkg, cuda, oracle, keys, off)


def test_cfg2_lengths_full_size(pkg, cuda, inst):
    """2^24 pairs in segments of 2^18 and 2^20 at the default threshold, the
    route on: sorted, stable, the values a permutation."""
    from test_parity_gpu import _u32_bits, assert_stable_sorted
    torch = cuda
    n = 1 << 24
    for lg in (18, 20):
        off = inst.equal_offsets(n, 1 << lg)
        keys = inst.uniform_keys(n, seed=lg + 300)
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


@pytest.mark.parametrize("kind", ["full_range", "two_digits", "narrow_top", "one_value"])
def test_u64_below_the_radix_threshold(pkg, cuda, oracle, inst, kind):
    """64-bit keys at the default thresholds: the MSD route takes segments
    above 2^15 although the radix threshold is 2^18; a segment that does not
    qualify (fewer than three varying digits, or a top digit that leaves long
    sub-buckets) is left to the merge passes of the second stage."""
    length = 40000
    n = 4 * length + 1234
    off = np.concatenate([inst.equal_offsets(4 * length, length), [n]]).astype(np.int32)
    keys = inst.uniform_keys(n, seed=77, bits=64, dtype=np.uint64)
    if kind == "two_digits":
        keys &= np.uint64(0xFFFF)
    elif kind == "narrow_top":
        # four varying digits, but the top one takes two values: sub-buckets
        # of about 20000 keys, longer than four tiles
        keys = ((keys >> np.uint64(63)) << np.uint64(56)) | (keys & np.uint64(0xFFFFFF))
    elif kind == "one_value":
        keys[:] = np.uint64(0x0123456789ABCDEF)
    with pkg.params({pkg.PARAM_MSD: 1}):
        check_both(pkg, cuda, oracle, keys, off)
