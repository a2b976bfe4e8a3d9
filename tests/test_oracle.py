"""CPU: the oracle is pinned against the reference before anything trusts it.

* the committed golden fixtures hold the reference's own outputs (its mseq
  program for keys, its gold_segsort for pairs; tests/golden/make_golden.py);
* where the reference programs are built here (oracle/_ref), the oracle is
  also compared with them live on fresh seeded instances;
* the C++ restatement and the numpy lexsort restatement agree;
* a mistake planted in a copy of the oracle's output is caught by the checks.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, load_golden


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_fixtures(oracle, name):
    g = load_golden(name)
    off, keys = g["offsets"], g["keys"]
    assert np.array_equal(oracle.segsort_cpp(keys, off), g["ref_keys"])
    assert np.array_equal(oracle.segsort_numpy(keys, off), g["ref_keys"])
    vals = np.arange(len(keys), dtype=np.uint32)
    k, v = oracle.segsort_cpp(keys, off, vals)
    assert np.array_equal(k, g["ref_pair_keys"]) and np.array_equal(v, g["ref_pair_vals"])
    k2, v2 = oracle.segsort_numpy(keys, off, vals)
    assert np.array_equal(k2, k) and np.array_equal(v2, v)


def test_golden_set_is_present():
    names = golden_cases()
    assert "ref_in1_32" in names and "ref_in2_1024" in names
    assert len(names) >= 10


@pytest.mark.skipif(not (__import__("oracle.oracle", fromlist=["x"]).REF_MSEQ.exists()),
                    reason="reference programs not built here (needs the reference checkout)")
@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_live_reference(oracle, inst, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 6000))
    nseg = int(rng.integers(1, min(n, 200) + 1))
    off = inst.diff_offsets(n, nseg, seed=100 + seed)
    bits = int(rng.choice([2, 12, 31]))
    keys = inst.uniform_keys(n, seed=200 + seed, bits=bits)
    assert np.array_equal(oracle.segsort_cpp(keys, off), oracle.run_reference_mseq(off, keys))


def test_cpp_and_numpy_agree_random(oracle, inst):
    rng = np.random.default_rng(7)
    for trial in range(20):
        n = int(rng.integers(0, 3000))
        cuts = np.sort(rng.integers(0, n + 1, int(rng.integers(0, 40))))
        off = np.concatenate([[0], cuts, [n]]).astype(np.int32)
        for dt in (np.uint32, np.int32, np.float32, np.uint64):
            if dt == np.float32:
                keys = rng.standard_normal(n).astype(np.float32)
                keys[rng.integers(0, max(n, 1), 5) % max(n, 1)] = 0.0 if n else 0.0
            else:
                keys = rng.integers(0, 8, n).astype(dt) * dt(3)
            vals = np.arange(n, dtype=np.uint32)
            k1, v1 = oracle.segsort_cpp(keys, off, vals, threads=3)
            k2, v2 = oracle.segsort_numpy(keys, off, vals)
            assert np.array_equal(k1.view(np.uint8), k2.view(np.uint8))
            assert np.array_equal(v1, v2)


def test_order_bits_semantics(oracle):
    f = np.array([np.nan, 1.0, -0.0, 0.0, -np.inf, np.inf, -1.0, -np.nan], dtype=np.float32)
    order = np.argsort(oracle.order_bits(f), kind="stable")
    got = f[order].view(np.uint32)
    # -NaN, -inf, -1, -0, +0, 1, +inf, +NaN
    exp = np.array([-np.nan, -np.inf, -1.0, -0.0, 0.0, 1.0, np.inf, np.nan],
                   dtype=np.float32).view(np.uint32)
    assert np.array_equal(got, exp)
    i = np.array([5, -3, 0, -2147483648, 2147483647], dtype=np.int32)
    assert np.array_equal(i[np.argsort(oracle.order_bits(i), kind="stable")],
                          np.sort(i))


def test_offsets_are_clamped_like_the_library(oracle):
    keys = np.array([9, 8, 7, 6, 5, 4], dtype=np.uint32)
    off = np.array([-5, 2, 100], dtype=np.int32)  # clamps to [0, 2), [2, 6)
    assert np.array_equal(oracle.segsort_cpp(keys, off), [8, 9, 4, 5, 6, 7])
    assert np.array_equal(oracle.segsort_numpy(keys, off), [8, 9, 4, 5, 6, 7])
    # a segment whose end is below its begin is empty; elements outside
    # every segment are untouched
    off = np.array([4, 1, 3], dtype=np.int32)
    assert np.array_equal(oracle.segsort_cpp(keys, off), [9, 7, 8, 6, 5, 4])
    assert np.array_equal(oracle.segsort_numpy(keys, off), [9, 7, 8, 6, 5, 4])


def test_heads_to_csr(oracle):
    assert list(oracle.heads_to_csr(np.array([0, 3, 3]), 10)) == [0, 3, 3, 10]


def test_planted_mistake_is_caught(oracle):
    """A checker that cannot fail proves nothing: swap two equal keys' values
    (an instability) and two keys (an unsorted pair) in a copy of the oracle's
    answer and check that the comparison used by the GPU tests rejects both."""
    g = load_golden("equal_len256_bits4")
    off, keys = g["offsets"], g["keys"]
    vals = np.arange(len(keys), dtype=np.uint32)
    k, v = oracle.segsort_cpp(keys, off, vals)
    i = int(np.flatnonzero(k[:-1] == k[1:])[0])
    v_bad = v.copy()
    v_bad[i], v_bad[i + 1] = v_bad[i + 1], v_bad[i]
    assert not np.array_equal(v_bad, g["ref_pair_vals"])
    j = int(np.flatnonzero(k[:-1] != k[1:])[0])
    k_bad = k.copy()
    k_bad[j], k_bad[j + 1] = k_bad[j + 1], k_bad[j]
    assert not np.array_equal(k_bad, g["ref_pair_keys"])


def test_oracle_descending_and_64bit_values(oracle):
    """The numpy restatement's descending mode against a plain Python stable
    sort by decreasing key, with 64-bit values carried along."""
    rng = np.random.default_rng(5)
    for dt in (np.uint32, np.int32, np.float32, np.uint64):
        n = 300
        if dt == np.float32:
            keys = rng.choice(np.array([-1.5, -0.0, 0.0, 2.0, 7.25], np.float32), n)
        else:
            keys = rng.integers(0, 6, n).astype(dt)
        off = np.array([0, 7, 7, 100, 101, 250, 300], np.int32)
        vals = rng.integers(0, 1 << 62, n, dtype=np.uint64)
        k, v = oracle.segsort_numpy(keys, off, vals, descending=True)
        ek, ev = keys.copy(), vals.copy()
        bits = oracle.order_bits(keys)
        for s in range(len(off) - 1):
            idx = list(range(off[s], off[s + 1]))
            idx = sorted(idx, key=lambda i: -int(bits[i]))  # stable
            ek[off[s]:off[s + 1]] = keys[idx]
            ev[off[s]:off[s + 1]] = vals[idx]
        assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)), dt
        assert v.dtype == np.uint64 and np.array_equal(v, ev), dt
