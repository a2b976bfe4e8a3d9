"""GPU parity of the tiny route (segments of a few keys), through the C ABI,
against the oracle.

Problems whose segments average at most SEGSORT_PARAM_TINY_MAX_AVG keys take
a persistent kernel that keeps two tiles' copies in flight and network-sorts
every chunk whose segments are at most 8 keys; other chunks (longer
segments, CAP-runs of long ones, a tile's later chunks) go to the fallback
list for the comparison sort.  Every case runs with the route forced on for
every multi-tile problem and off.  Bar: bit-exact keys and values, stable
order of equal keys included.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_parity_gpu import check_both

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["tiny", "off"])
def route(request, pkg, cuda):
    if request.param == "tiny":
        p = {pkg.PARAM_TINY_MAX_AVG: 1 << 30, pkg.PARAM_STREAM_MAX_AVG: 1 << 30}
    else:
        p = {pkg.PARAM_TINY_MAX_AVG: 0}
    with pkg.params(p):
        yield request.param


@pytest.mark.parametrize("length", [1, 2, 3, 4, 5, 7, 8, 9, 12, 16, 17, 31, 33, 40, 63, 64, 65])
@pytest.mark.parametrize("bits", [32, 2])
def test_equal_segments(pkg, cuda, oracle, inst, route, length, bits):
    n = 100003 // length * length + length // 2  # ragged last segment
    off = np.concatenate([inst.equal_offsets(n - length // 2, length), [n]]).astype(np.int32)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=length * 11 + bits, bits=bits), off)


def test_random_short_and_some_long(pkg, cuda, oracle, inst, route):
    rng = np.random.default_rng(121)
    lens = rng.integers(0, 9, 60000)
    lens[::5000] = rng.integers(9, 300, len(lens[::5000]))  # chunks the tiny kernel lists
    lens[7777] = 50000                                       # a long segment: CAP-runs and merges
    lens[33333] = 9000
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=122), off)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=123, bits=3), off)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=124), off[:-1], heads=True)


def test_lognormal_small_mean(pkg, cuda, oracle, inst, route):
    off = inst.lognormal_offsets(1 << 19, seed=125, mu=1.0, sigma=1.2, empty_frac=0.05)
    check_both(pkg, cuda, oracle, inst.uniform_keys(1 << 19, seed=125), off)
    check_both(pkg, cuda, oracle, inst.zipf_keys(1 << 19, seed=126), off)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_key_types(pkg, cuda, oracle, inst, route, dtype):
    rng = np.random.default_rng(127)
    lens = rng.integers(1, 9, 30000)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 10).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-42, -1e-42], np.float32)
        keys[rng.integers(0, n, 3000)] = specials[rng.integers(0, len(specials), 3000)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=128).view(np.int32).copy()
        keys[::7] = np.int32(-2147483648)
        keys[::13] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=129, bits=64, dtype=np.uint64)
        keys[::3] &= np.uint64(0xFF)
    check_both(pkg, cuda, oracle, keys, off)


def test_presorted_and_mixed(pkg, cuda, oracle, inst, route):
    """Chunks whose keys are already in order go back unwritten; the others
    around them are still sorted (the decision is per chunk)."""
    rng = np.random.default_rng(130)
    lens = rng.integers(1, 9, 40000)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    check_both(pkg, cuda, oracle, np.arange(n, dtype=np.uint32), off)
    keys = np.arange(n, dtype=np.uint32)
    keys[n // 3: 2 * n // 3] = inst.uniform_keys(2 * n // 3 - n // 3, seed=131)
    check_both(pkg, cuda, oracle, keys, off)
    eq = np.full(n, 7, dtype=np.uint32)  # equal keys: the stable order is the input order
    check_both(pkg, cuda, oracle, eq, off)


@pytest.mark.parametrize("top", [8, 16, 64])
def test_random_lengths_up_to(pkg, cuda, oracle, inst, route, top):
    """Lengths spread over [0, top]: with top 8 every chunk is sorted by the
    networks, above it most chunks go to the list (empty segments, single
    keys and every length below top included)."""
    rng = np.random.default_rng(140 + top)
    lens = rng.integers(0, top + 1, 200000 // top)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=141 + top), off)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=142 + top, bits=3), off)
