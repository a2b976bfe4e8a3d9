"""GPU parity: the CUDA path, called through the C ABI, against the oracle.

Bar: bit-exact keys and values (integer work), including the stable order of
equal keys.  Small and mid sizes compare element by element with the oracle
(and with the reference's own outputs in tests/golden/).  Full benchmark
sizes use properties that together imply equality with the stable sort:
every output position holds an input position of its own segment exactly
once (a permutation per segment), keys moved with their values, keys are
non-decreasing within a segment, and equal keys keep increasing input
positions (stability).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

_SUFFIX = {np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32",
           np.dtype(np.float32): "f32", np.dtype(np.uint64): "u64"}
_VIEW = {np.dtype(np.uint32): np.int32, np.dtype(np.int32): np.int32,
         np.dtype(np.float32): np.float32, np.dtype(np.uint64): np.int64}
GUARD = 3  # elements of guard band on each side (also makes the pointers unaligned)


def _dev(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(_VIEW[arr.dtype])).cuda()


def gpu_sort(pkg, torch, keys, off, vals=None, heads=False, ws=None):
    """Sort through the C ABI with guard bands around the data; returns the
    sorted numpy arrays and checks the guards were not touched."""
    L = pkg.lib()
    suf = _SUFFIX[keys.dtype]
    n = len(keys)
    sentinel_k = np.full(GUARD, 0x5A, dtype=keys.dtype)
    kbuf = _dev(torch, np.concatenate([sentinel_k, keys, sentinel_k]))
    kptr = kbuf.data_ptr() + GUARD * keys.itemsize
    vbuf = vptr = None
    if vals is not None:
        sentinel_v = np.full(GUARD, 0xA5A5A5A5, dtype=np.uint32)
        vbuf = _dev(torch, np.concatenate([sentinel_v, vals, sentinel_v]))
        vptr = vbuf.data_ptr() + GUARD * 4
    dof = torch.from_numpy(np.ascontiguousarray(off, dtype=np.int32)).cuda()
    nseg = len(off) - (0 if heads else 1)
    st = torch.cuda.current_stream().cuda_stream
    if ws is not None:
        wsb = torch.empty(ws, dtype=torch.uint8, device="cuda")
        if vals is None:
            rc = L.segsort_keys_u32_ws(kptr, n, dof.data_ptr(), nseg, wsb.data_ptr(), ws, st)
        else:
            rc = L.segsort_pairs_u32_ws(kptr, vptr, n, dof.data_ptr(), nseg, wsb.data_ptr(), ws, st)
    elif heads:
        rc = (L.segsort_keys_u32_heads(kptr, n, dof.data_ptr(), nseg, st) if vals is None else
              L.segsort_pairs_u32_heads(kptr, vptr, n, dof.data_ptr(), nseg, st))
    elif vals is None:
        rc = getattr(L, f"segsort_keys_{suf}")(kptr, n, dof.data_ptr(), nseg, st)
    else:
        rc = getattr(L, f"segsort_pairs_{suf}")(kptr, vptr, n, dof.data_ptr(), nseg, st)
    assert rc == pkg.SEGSORT_OK, L.segsort_error_string(rc)
    torch.cuda.synchronize()
    assert pkg.device_status() == pkg.SEGSORT_OK
    kout = kbuf.cpu().numpy().view(keys.dtype)
    assert np.array_equal(kout[:GUARD].view(np.uint8), sentinel_k.view(np.uint8))
    assert np.array_equal(kout[GUARD + n:].view(np.uint8), sentinel_k.view(np.uint8))
    if vals is None:
        return kout[GUARD:GUARD + n].copy()
    vout = vbuf.cpu().numpy().view(np.uint32)
    assert np.array_equal(vout[:GUARD], sentinel_v) and np.array_equal(vout[GUARD + n:], sentinel_v)
    return kout[GUARD:GUARD + n].copy(), vout[GUARD:GUARD + n].copy()


def same_bits(a, b) -> bool:
    return a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def check_both(pkg, torch, oracle, keys, off, heads=False):
    """Keys-only and pairs (values = input index) against the numpy oracle."""
    csr = oracle.heads_to_csr(off, len(keys)) if heads else off
    exp_k = oracle.segsort_numpy(keys, csr)
    got_k = gpu_sort(pkg, torch, keys, off, heads=heads)
    assert same_bits(got_k, exp_k), first_diff(got_k, exp_k)
    vals = np.arange(len(keys), dtype=np.uint32)
    exp_k2, exp_v = oracle.segsort_numpy(keys, csr, vals)
    got_k2, got_v = gpu_sort(pkg, torch, keys, off, vals, heads=heads)
    assert same_bits(got_k2, exp_k2), first_diff(got_k2, exp_k2)
    assert np.array_equal(got_v, exp_v), first_diff(got_v, exp_v)


def first_diff(a, b) -> str:
    ab = a.view(np.uint8).reshape(len(a), -1)
    bb = b.view(np.uint8).reshape(len(b), -1)
    bad = np.flatnonzero(np.any(ab != bb, axis=1))
    if len(bad) == 0:
        return "equal"
    i = int(bad[0])
    return f"{len(bad)} mismatches, first at {i}: got {a[i]} expected {b[i]}"


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", golden_cases())
def test_reference_fixtures(pkg, cuda, name):
    g = load_golden(name)
    off, keys = g["offsets"], g["keys"]
    assert np.array_equal(gpu_sort(pkg, cuda, keys, off), g["ref_keys"])
    k, v = gpu_sort(pkg, cuda, keys, off, np.arange(len(keys), dtype=np.uint32))
    assert np.array_equal(k, g["ref_pair_keys"])
    assert np.array_equal(v, g["ref_pair_vals"])


def test_every_length_up_to_700(pkg, cuda, oracle, inst):
    rng = np.random.default_rng(1)
    lens = np.repeat(np.arange(0, 701), 2)
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    for bits in (32, 3):
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=bits, bits=bits), off)


@pytest.mark.parametrize("length", list(range(1, 34)) + [63, 64, 65, 127, 128, 129, 255, 256,
                                                        257, 511, 512, 513, 1000, 1023, 1024,
                                                        1025, 2047, 2048, 2049, 3000, 4095,
                                                        4096, 4097, 5000, 8191, 8192, 8193,
                                                        12289, 65536, 100000])
def test_equal_segments(pkg, cuda, oracle, inst, length):
    n = max(length * 3, 1 << 16) // length * length + (length // 3)  # ragged tail segment
    off = np.concatenate([inst.equal_offsets(n - length // 3, length), [n]]).astype(np.int32)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=length, bits=32), off)


@pytest.mark.parametrize("bits", [0, 1, 4, 12])
def test_low_entropy_stability(pkg, cuda, oracle, inst, bits):
    off = inst.lognormal_offsets(1 << 18, seed=bits + 40, empty_frac=0.05)
    keys = (inst.uniform_keys(1 << 18, seed=bits, bits=max(bits, 1))
            if bits else np.zeros(1 << 18, np.uint32))
    check_both(pkg, cuda, oracle, keys, off)


def test_random_cut_segments(pkg, cuda, oracle, inst):
    for nseg, n, seed in [(1, 50000, 1), (7, 100000, 2), (300, 200000, 3), (30000, 100000, 4)]:
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=seed), inst.diff_offsets(n, nseg, seed))


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_key_types(pkg, cuda, oracle, inst, dtype):
    rng = np.random.default_rng(5)
    lens = [0, 1, 2, 3, 17, 100, 1000, 2047, 2048, 2049, 4096, 4097, 9000, 30000, 5, 0]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 1e3).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 1e-42, -1e-42,
                             np.finfo(np.float32).max, -np.finfo(np.float32).max], np.float32)
        keys[rng.integers(0, n, 400)] = specials[rng.integers(0, len(specials), 400)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=9).view(np.int32).copy()
        keys[::11] = np.int32(-2147483648)
        keys[::13] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=10, bits=64, dtype=np.uint64)
        keys[::5] &= np.uint64(0xFFFF)  # equal low halves: compare across both words
        keys[::17] = np.uint64(0xFFFFFFFFFFFFFFFF)
    check_both(pkg, cuda, oracle, keys, off)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64])
def test_short_segment_key_types(pkg, cuda, oracle, inst, dtype):
    """Every key type on problems of short ragged segments (average below 32,
    over many tiles: the streamed tile kernel and the half-tile classify),
    with a few long segments among them."""
    rng = np.random.default_rng(31)
    lens = rng.integers(0, 20, 6000)
    lens[::1500] = [5000, 9000, 4097, 12000]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    assert n < 32 * (len(off) - 1)
    if dtype == np.float32:
        keys = (rng.standard_normal(n) * 10).astype(np.float32)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-42, -1e-42], np.float32)
        keys[rng.integers(0, n, 500)] = specials[rng.integers(0, len(specials), 500)]
    elif dtype == np.int32:
        keys = inst.uniform_keys(n, seed=32, bits=6).astype(np.int32) - 32
        keys[::13] = np.int32(-2147483648)
        keys[::17] = 2147483647
    else:
        keys = inst.uniform_keys(n, seed=33, bits=64, dtype=np.uint64)
        keys[::3] &= np.uint64(0xFF)
    check_both(pkg, cuda, oracle, keys, off)


def test_heads_only_offsets(pkg, cuda, oracle, inst):
    n = 60000
    csr = inst.diff_offsets(n, 50, seed=11)
    keys = inst.uniform_keys(n, seed=11, bits=10)
    check_both(pkg, cuda, oracle, keys, csr[:-1], heads=True)


def test_caller_workspace(pkg, cuda, oracle, inst):
    n = 300000
    off = inst.diff_offsets(n, 20, seed=12)
    keys = inst.uniform_keys(n, seed=12)
    vals = np.arange(n, dtype=np.uint32)
    ws = pkg.workspace_bytes(n, 20, 4, 4)
    assert ws > 0
    k, v = gpu_sort(pkg, cuda, keys, off, vals, ws=ws)
    ek, ev = oracle.segsort_numpy(keys, off, vals)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)
    k = gpu_sort(pkg, cuda, keys, off, ws=pkg.workspace_bytes(n, 20, 4, 0))
    assert np.array_equal(k, oracle.segsort_numpy(keys, off))
    # too small a workspace is refused before anything runs
    L = pkg.lib()
    buf = cuda.empty(16, dtype=cuda.uint8, device="cuda")
    d = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    o = cuda.from_numpy(off).cuda()
    assert L.segsort_keys_u32_ws(d.data_ptr(), n, o.data_ptr(), 20, buf.data_ptr(), 16,
                                 cuda.cuda.current_stream().cuda_stream) == pkg.SEGSORT_ERR_WORKSPACE


def test_edge_cases(pkg, cuda, oracle, inst):
    k1 = np.array([7], np.uint32)
    check_both(pkg, cuda, oracle, k1, np.array([0, 1], np.int32))
    # nothing covered: offsets leave a prefix and a suffix untouched
    keys = inst.uniform_keys(20000, seed=13)
    check_both(pkg, cuda, oracle, keys, np.array([100, 5000, 5000, 19001], np.int32))
    # all segments empty
    check_both(pkg, cuda, oracle, keys[:10], np.array([0, 0, 0, 0], np.int32))
    # thousands of empty segments at one position, between short ones
    lens = np.zeros(6000, np.int64)
    lens[::500] = np.arange(12) * 37 + 1
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    check_both(pkg, cuda, oracle, inst.uniform_keys(int(off[-1]), seed=14, bits=5), off)
    # maximum keys everywhere (they equal no padding value in the words)
    kmax = np.full(10000, 0xFFFFFFFF, np.uint32)
    kmax[::3] = 0
    check_both(pkg, cuda, oracle, kmax, np.array([0, 9, 4100, 10000], np.int32))
    # already sorted and reverse sorted input
    s = np.sort(inst.uniform_keys(50000, seed=15))
    check_both(pkg, cuda, oracle, s, inst.diff_offsets(50000, 9, 15))
    check_both(pkg, cuda, oracle, s[::-1].copy(), inst.diff_offsets(50000, 9, 16))
    # offsets out of [0, n] are clamped (monotone after clamping)
    check_both(pkg, cuda, oracle, keys[:9000], np.array([-50, 3000, 8000, 123456], np.int32))


def test_keys_and_values_aligned_differently(pkg, cuda, oracle, inst):
    """Keys and values at different offsets from a 16-byte boundary, over many
    tiles: each array's staged middle and ragged ends are found separately."""
    torch = cuda
    L = pkg.lib()
    n = 50000
    st = torch.cuda.current_stream().cuda_stream
    for kshift, vshift in ((1, 2), (3, 0), (0, 1), (2, 3)):
        for off in (inst.lognormal_offsets(n, seed=20 + kshift, empty_frac=0.05),
                    inst.equal_offsets_ragged(n, 7 + kshift * 300)):
            keys = inst.uniform_keys(n, seed=30 + kshift, bits=12)
            vals = np.arange(n, dtype=np.uint32)
            kb = torch.full((n + 8,), -1, dtype=torch.int32, device="cuda")
            vb = torch.full((n + 8,), -2, dtype=torch.int32, device="cuda")
            kb[kshift:kshift + n] = torch.from_numpy(keys.view(np.int32)).cuda()
            vb[vshift:vshift + n] = torch.from_numpy(vals.view(np.int32)).cuda()
            dof = torch.from_numpy(off).cuda()
            rc = L.segsort_pairs_u32(kb.data_ptr() + 4 * kshift, vb.data_ptr() + 4 * vshift, n,
                                     dof.data_ptr(), len(off) - 1, st)
            assert rc == pkg.SEGSORT_OK
            torch.cuda.synchronize()
            assert pkg.device_status() == pkg.SEGSORT_OK
            k = kb.cpu().numpy().view(np.uint32)
            v = vb.cpu().numpy().view(np.uint32)
            ek, ev = oracle.segsort_numpy(keys, off, vals)
            assert np.array_equal(k[kshift:kshift + n], ek), first_diff(k[kshift:kshift + n], ek)
            assert np.array_equal(v[vshift:vshift + n], ev), first_diff(v[vshift:vshift + n], ev)
            assert np.all(k[:kshift] == 0xFFFFFFFF) and np.all(k[kshift + n:] == 0xFFFFFFFF)
            assert np.all(v[:vshift] == 0xFFFFFFFE) and np.all(v[vshift + n:] == 0xFFFFFFFE)


def test_dense_segment_starts_across_tiles(pkg, cuda, oracle, inst):
    """Tiles whose chunks hold more segment starts than elements: runs of
    length-1 segments and thousands of empty segments inside a multi-tile
    problem, between short and long ones."""
    rng = np.random.default_rng(21)
    lens = np.concatenate([np.ones(10000), np.zeros(5000), rng.integers(0, 9, 8000),
                           np.zeros(3000), [9000], np.full(2000, 3), np.zeros(4500), [2],
                           np.ones(6000)]).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    for bits in (32, 2):
        check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=22 + bits, bits=bits), off)
    check_both(pkg, cuda, oracle, inst.uniform_keys(n, seed=23, bits=5), off[:-1], heads=True)


@pytest.mark.parametrize("dtype,block", [(np.uint32, 16), (np.uint64, 8)])
def test_segments_within_thread_blocks(pkg, cuda, oracle, inst, dtype, block):
    """Every block of `block` positions (one thread's words in the tile sort)
    split into segments of 1..12 elements: no segment crosses a block, so
    the tile sort uses no merge level and sorts each block's segments in
    registers (transposition rounds up to the longest segment, or the
    bitonic network)."""
    rng = np.random.default_rng(block)
    lens = []
    for _ in range(40000 // block):
        left = block
        while left:
            ln = int(min(left, rng.integers(1, 13)))
            lens.append(ln)
            left -= ln
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    n = int(off[-1])
    for bits in (3, 32):
        keys = inst.uniform_keys(n, seed=40 + bits, bits=bits, dtype=dtype)
        check_both(pkg, cuda, oracle, keys, off)


def test_repeated_calls_are_idempotent(pkg, cuda, oracle, inst):
    n = 1 << 17
    off = inst.lognormal_offsets(n, seed=17)
    keys = inst.uniform_keys(n, seed=17, bits=8)
    vals = np.arange(n, dtype=np.uint32)
    k, v = gpu_sort(pkg, cuda, keys, off, vals)
    k2, v2 = gpu_sort(pkg, cuda, k, off, v)
    assert np.array_equal(k, k2) and np.array_equal(v, v2)


def test_cfg1_keys_only_2e20_1024_segments(pkg, cuda, oracle, inst):
    n = 1 << 20
    keys = inst.uniform_keys(n, seed=1, bits=31)
    off = inst.equal_offsets(n, 1024)
    assert np.array_equal(gpu_sort(pkg, cuda, keys, off), oracle.segsort_cpp(keys, off, threads=8))


# ---------------------------------------------------------------------------
# Full-size properties.
def assert_stable_sorted(torch, bits_in, bits_out, vals_out, off_np):
    """bits_* int64 tensors of order bits; vals_out int64 input positions."""
    dev = bits_in.device
    n = bits_in.numel()
    off = torch.from_numpy(np.clip(off_np.astype(np.int64), 0, n)).to(dev)
    lens = (off[1:] - off[:-1]).clamp(min=0)
    seg = torch.repeat_interleave(torch.arange(len(lens), device=dev), lens)
    first = torch.repeat_interleave(off[:-1], lens)
    rank = torch.arange(seg.numel(), device=dev) - torch.repeat_interleave(torch.cumsum(lens, 0) - lens, lens)
    pos = first + rank
    v = vals_out[pos]
    assert bool(((v >= off[:-1][seg]) & (v < off[1:][seg])).all()), "value outside its segment"
    cnt = torch.bincount(v, minlength=n)
    assert bool((cnt[pos] == 1).all()), "values are not a permutation of the segment"
    k = bits_out[pos]
    assert torch.equal(bits_in[v], k), "keys did not move with their values"
    same = seg[1:] == seg[:-1]
    assert bool((~same | (k[:-1] <= k[1:])).all()), "not sorted"
    assert bool((~same | (k[:-1] != k[1:]) | (v[:-1] < v[1:])).all()), "not stable"


def sort_on_device_u32(pkg, torch, dk, dv, off_np):
    dof = torch.from_numpy(off_np).cuda()
    rc = pkg.lib().segsort_pairs_u32(dk.data_ptr(), dv.data_ptr(), dk.numel(), dof.data_ptr(),
                                     len(off_np) - 1, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert pkg.device_status() == 0


def _u32_bits(t):
    return t.long() & 0xFFFFFFFF


@pytest.mark.parametrize("log_len", range(1, 21))
def test_cfg2_equal_segments_2e24_pairs(pkg, cuda, inst, log_len):
    torch = cuda
    n = 1 << 24
    off = inst.equal_offsets(n, 1 << log_len)
    for bits in (32, 4):
        keys = inst.uniform_keys(n, seed=log_len, bits=bits)
        dk = torch.from_numpy(keys.view(np.int32)).cuda()
        before = _u32_bits(dk)
        dv = torch.arange(n, dtype=torch.int32, device="cuda")
        sort_on_device_u32(pkg, torch, dk, dv, off)
        assert_stable_sorted(torch, before, _u32_bits(dk), dv.long(), off)


@pytest.mark.parametrize("keys_kind", ["uniform", "zipf"])
def test_cfg3_lognormal_2e25_pairs(pkg, cuda, inst, oracle, keys_kind):
    torch = cuda
    n = 1 << 25
    off = inst.lognormal_offsets(n, seed=3)
    keys = inst.uniform_keys(n, seed=3) if keys_kind == "uniform" else inst.zipf_keys(n, seed=3)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    before = _u32_bits(dk)
    dv = torch.arange(n, dtype=torch.int32, device="cuda")
    sort_on_device_u32(pkg, torch, dk, dv, off)
    assert_stable_sorted(torch, before, _u32_bits(dk), dv.long(), off)
    # and element by element against the oracle on this full instance
    ek, ev = oracle.segsort_numpy(keys, off, np.arange(n, dtype=np.uint32))
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), ek)
    assert np.array_equal(dv.cpu().numpy().view(np.uint32), ev)


def test_device_status_is_clean(pkg, cuda):
    assert pkg.device_status() == pkg.SEGSORT_OK
