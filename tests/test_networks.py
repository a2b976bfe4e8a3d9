"""CPU checks of the combinatorial facts the sort kernels rely on.

* Batcher's odd-even merge network, enumerated by the same loop nest as
  BatcherNet<N>::pair (segmented-sorting_gb300/csrc/tile_sort.cuh), sorts
  every 0-1 input of 4, 8 and 16 words (so every input, by the 0-1
  principle) with 5, 19 and 63 compare-exchanges, each (low, high).
* R rounds of odd-even transposition sort any run of at most R words,
  whichever parity the run's first position has (transposition_sort).
* The half-tile classify (one lower-bound search per half-tile entry and one
  long-segment candidate per half-tile, large_classify_halves_kernel in
  csrc/classify.cuh) writes the same half-tile map and job list as the
  per-boundary classify (classify_boundary).
* The streamed tile kernel's staging geometry (StagedSpan in
  csrc/tile_stream.cuh): the bulk copy starts on a 16-byte boundary inside
  the range's first granule, covers every element, and stays inside the
  staging buffer (CAP + 32 / sizeof(T) elements, CAP/2 + 8 for offsets).
* The tiny route's networks (tiny_sort_segment in csrc/tiny_sort.cuh, read
  from the source) sort every 0-1 input of 2, 4 and 8 words with 1, 5 and 19
  comparators, and over (order bits, slot) composites with padded slots give
  the stable order; store_staged writes every element of a chunk exactly
  once whatever its misalignment; its kernel's schedule of plans, copies
  and barrier phases (restated) never reads a plan or stage early or late.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest


def batcher_pairs(n: int) -> list[tuple[int, int]]:
    out = []
    p = 1
    while p < n:
        k = p
        while k >= 1:
            j = k % p
            while j + k < n:
                for i in range(min(k, n - j - k)):
                    if (i + j) // (2 * p) == (i + j + k) // (2 * p):
                        out.append((i + j, i + j + k))
                j += 2 * k
            k //= 2
        p *= 2
    return out


def zero_one_inputs(n: int) -> np.ndarray:
    return np.array(list(itertools.product([0, 1], repeat=n)), dtype=np.int8)


@pytest.mark.parametrize("n,size", [(4, 5), (8, 19), (16, 63)])
def test_batcher_network_sorts_every_input(n, size):
    pairs = batcher_pairs(n)
    assert len(pairs) == size and all(a < b for a, b in pairs)
    x = zero_one_inputs(n)
    for a, b in pairs:
        lo = np.minimum(x[:, a], x[:, b])
        hi = np.maximum(x[:, a], x[:, b])
        x[:, a], x[:, b] = lo, hi
    assert np.all(np.diff(x, axis=1) >= 0)


@pytest.mark.parametrize("length", list(range(1, 17)))
def test_transposition_rounds_sort_runs_of_their_length(length):
    x0 = zero_one_inputs(length)
    for parity in (0, 1):
        x = x0.copy()
        for r in range(length):
            for i in range((r + parity) % 2, length - 1, 2):
                lo = np.minimum(x[:, i], x[:, i + 1])
                hi = np.maximum(x[:, i], x[:, i + 1])
                x[:, i], x[:, i + 1] = lo, hi
        assert np.all(np.diff(x, axis=1) >= 0), (length, parity)


def _off(o, nseg, i, n):
    return min(max(int(o[i]), 0), n)


def _lower_bound(o, nseg, n, x):
    """The warp's 32-ary search of warp_lower_bound, one probe set per round."""
    lo, hi = 0, nseg
    while hi > lo:
        span = hi - lo
        small = span <= 32
        probes = [lo + l if small else lo + (span * (l + 1)) // 33 for l in range(32)]
        ge = [True if (small and l >= span) else _off(o, nseg, probes[l], n) >= x
              for l in range(32)]
        c = sum(1 for g in ge if not g)
        assert ge == [False] * c + [True] * (32 - c)  # a monotone ballot
        if small:
            lo += c
            hi = lo
        else:
            lo, hi = (probes[c - 1] + 1 if c > 0 else lo), (probes[c] if c < 32 else hi)
    return lo


def test_half_tile_classify_matches_per_boundary_classify():
    rng = np.random.default_rng(0)
    cap, half = 4096, 2048
    for trial in range(48):
        nseg = int(rng.integers(1, 2500))
        kind = trial % 4
        if kind == 0:
            lens = rng.integers(0, 5, nseg)
        elif kind == 1:
            lens = rng.integers(0, 9000, nseg) * (rng.random(nseg) < 0.3)
        elif kind == 2:
            lens = np.where(rng.random(nseg) < 0.01, rng.integers(4097, 20000, nseg),
                            rng.integers(0, 3, nseg))
        else:
            lens = rng.integers(1, 100, nseg)
        o = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        n = int(o[-1]) + int(rng.integers(0, 50))
        halves = 2 * max(1, (n + cap - 1) // cap)
        # per-boundary definition: boundary s owns the entries h with
        # off(s-1) < h*half <= off(s) (off(-1) = -inf, off(nseg) = +inf)
        ref = [None] * (halves + 1)
        for s in range(nseg + 1):
            cur = _off(o, nseg, s, n) if s < nseg else 0
            h_lo = 0 if s == 0 else _off(o, nseg, s - 1, n) // half + 1
            h_hi = halves if s == nseg else min(cur // half, halves)
            for h in range(h_lo, h_hi + 1):
                ref[h] = s
        jobs_ref = sorted((_off(o, nseg, s, n), _off(o, nseg, s + 1, n)) for s in range(nseg)
                          if _off(o, nseg, s + 1, n) - _off(o, nseg, s, n) > cap)
        hf = [_lower_bound(o, nseg, n, h * half) for h in range(halves + 1)]
        assert hf == ref, trial
        jobs = []
        for h in range(halves):
            if hf[h + 1] > hf[h]:
                beg, end = _off(o, nseg, hf[h + 1] - 1, n), _off(o, nseg, hf[h + 1], n)
                if end - beg > cap:
                    jobs.append((beg, end))
        assert sorted(jobs) == jobs_ref, trial


@pytest.mark.parametrize("elem", [4, 8])
def test_staged_span_geometry(elem):
    cap = 4096 if elem == 4 else 2048
    v = 16 // elem
    for stage_cap, limit in ((cap + 32 // elem, cap), (cap // 2 + 8, cap // 2)):
        for addr_elems in range(0, 2 * v):       # the range's first element, in elements
            for m in list(range(1, 40)) + [limit - 1, limit]:
                byte0 = addr_elems * elem
                mis = (byte0 & 15) // elem
                nvec = (mis + m + v - 1) // v
                copy_from = byte0 - mis * elem   # the bulk copy's global start
                assert copy_from % 16 == 0 and copy_from >= (byte0 // 16) * 16
                assert mis + m <= nvec * v       # every element is copied
                assert nvec * v <= stage_cap     # inside the staging buffer
                # the last granule holds the range's last element (no granule past it)
                assert (copy_from + 16 * nvec) - (byte0 + m * elem) < 16


# ---------------------------------------------------------------------------
# The tiny route (csrc/tiny_sort.cuh): the comparators of tiny_sort_segment
# are read from the source, so the check covers the networks the kernel runs.
TINY_SRC = (__import__("pathlib").Path(__file__).resolve().parents[1]
            / "segmented-sorting_gb300" / "csrc" / "tiny_sort.cuh")


def tiny_networks() -> dict[int, list[tuple[int, int]]]:
    import re
    src = TINY_SRC.read_text()
    body = src[src.index("bool tiny_sort_segment("):]
    body = body[body.index("if constexpr (N == 2) {"):body.index("// Two keys")]
    n2, rest = body.split("} else if constexpr (N == 4) {")
    n4, n8 = rest.split("} else {")
    pat = re.compile(r"W::cx\(w\[(\d+)\], w\[(\d+)\]\)")
    return {n: [(int(a), int(b)) for a, b in pat.findall(part)]
            for n, part in ((2, n2), (4, n4), (8, n8))}


@pytest.mark.parametrize("n,size", [(2, 1), (4, 5), (8, 19)])
def test_tiny_networks_sort_every_input(n, size):
    pairs = tiny_networks()[n]
    assert len(pairs) == size and all(a < b < n for a, b in pairs)
    x = zero_one_inputs(n)
    for a, b in pairs:
        lo = np.minimum(x[:, a], x[:, b])
        hi = np.maximum(x[:, a], x[:, b])
        x[:, a], x[:, b] = lo, hi
    assert np.all(np.diff(x, axis=1) >= 0)


@pytest.mark.parametrize("n", [2, 4, 8])
def test_tiny_composites_give_the_stable_order(n):
    """Every segment length up to the network's width: (order bits << 6 | slot)
    composites, the slots past the segment padded with the largest value, come
    out as the stable order of the keys (few distinct keys: many ties)."""
    pairs = tiny_networks()[n]
    rng = np.random.default_rng(7 + n)
    pad = (1 << 64) - 1
    for length in range(1, n + 1):
        for _ in range(300):
            keys = [int(k) for k in rng.integers(0, 3, length)]
            keys[0] = (1 << 32) - 1 if rng.random() < 0.2 else keys[0]  # the largest key too
            w = [(k << 6) | q for q, k in enumerate(keys)] + [pad] * (n - length)
            for a, b in pairs:
                if w[a] > w[b]:
                    w[a], w[b] = w[b], w[a]
            got = [(x >> 6, x & 63) for x in w[:length]]
            want = sorted(((k, q) for q, k in enumerate(keys)), key=lambda t: t[0])  # stable
            assert got == want and all(x == pad for x in w[length:])


@pytest.mark.parametrize("elem", [4, 8])
def test_store_staged_writes_each_element_once(elem):
    """store_staged's split of [0, m) into whole 16-byte granules and the
    ragged head and tail, restated: every element is written exactly once and
    nothing outside [0, m), for every misalignment, chunk size and block size."""
    e = 16 // elem
    for nt in (32, 512):
        for mis in range(e):
            for m in list(range(0, 70)) + [2047, 2048, 4095, 4096]:
                writes = [0] * (m + 2 * e)  # index i + e is element i
                g0, g1 = (mis + e - 1) // e, (mis + m) // e
                if g1 > g0:
                    for g in range(g0, g1):            # granule g covers elements g*e - mis ..
                        for c in range(e):
                            writes[g * e - mis + c + e] += 1
                    h, t = g0 * e - mis, g1 * e - mis
                    for tid in range(nt):
                        if tid < h:
                            writes[tid + e] += 1
                        if tid < m - t:
                            writes[t + tid + e] += 1
                else:
                    for i in range(m):
                        writes[i + e] += 1
                assert writes[e:e + m] == [1] * m, (nt, mis, m)
                assert sum(writes) == m, (nt, mis, m)


@pytest.mark.parametrize("iters", list(range(1, 40)) + [64, 100])
def test_tiny_kernel_schedule(iters):
    """tile_tiny_kernel's schedule, restated: plans made kPlanBatch (16) at a
    time into a ring of kPlanRing (32) by warp 0, copies of iteration i into
    stage i & 1 issued two iterations ahead, the wait of iteration i on its
    stage's barrier with parity (i >> 1) & 1.  Every plan is written before
    the copy or the sort that reads it and is not overwritten while either
    still needs it; every wait expects the phase its stage is in; a stage is
    refilled only after the sort of its previous tile has ended."""
    batch, ring = 16, 32
    slot_of = {}                      # ring slot -> iteration whose plan it holds
    phases = [0, 0]                   # completed phases per stage barrier
    in_flight = [None, None]          # iteration whose copy is in each stage

    def make_plans(i0):
        for i in range(i0, min(i0 + batch, iters)):
            slot_of[i % ring] = i

    def issue(i):
        assert slot_of.get(i % ring) == i          # its plan is there
        assert in_flight[i & 1] is None            # the stage is free
        in_flight[i & 1] = i

    make_plans(0)
    issue(0)
    if iters > 1:
        issue(1)
    for i in range(iters):
        s = i & 1
        assert in_flight[s] == i
        assert phases[s] % 2 == (i >> 1) & 1       # the parity the wait expects
        phases[s] += 1                             # the copy completes the phase
        assert slot_of.get(i % ring) == i          # the sort reads its plan
        in_flight[s] = None                        # end-of-iteration barrier: stage free
        if i + 2 < iters:
            if (i + 2) % batch == 0:
                # the batch overwrites slots (i+2 .. i+17) % 32: none still needed
                needed = {j % ring for j in (i + 1,) if j < iters}
                assert not needed & {j % ring for j in range(i + 2, min(i + 2 + batch, iters))}
                make_plans(i + 2)
            issue(i + 2)
    assert in_flight == [None, None]               # no copy outstanding at the end
