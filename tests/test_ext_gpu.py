"""GPU parity of the extensions: stable descending order, segmented top-k,
64-bit values and segmented reduce-by-key, through the C ABI, bit for bit
against the oracle (numpy restatement with descending=True / 64-bit values,
and a Python loop over the oracle's sorted runs), with guard bands around
the buffers of the in-place forms."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_VIEW = {np.dtype(np.uint32): np.int32, np.dtype(np.int32): np.int32,
         np.dtype(np.float32): np.float32, np.dtype(np.uint64): np.int64}
_SUF = {np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32",
        np.dtype(np.float32): "f32", np.dtype(np.uint64): "u64"}
G = 3  # guard elements


def _guarded(torch, a, fill):
    g = np.full(G, fill, dtype=a.dtype)
    t = torch.from_numpy(np.concatenate([g, a, g]).view(_VIEW[a.dtype] if a.dtype in _VIEW
                                                        else np.int64)).cuda()
    return t, g


def _unguard(t, dtype, n, g):
    a = t.cpu().numpy().view(dtype)
    assert np.array_equal(a[:G].view(np.uint8), g.view(np.uint8))
    assert np.array_equal(a[G + n:].view(np.uint8), g.view(np.uint8))
    return a[G:G + n].copy()


def _instances(inst):
    out = []
    for t in ("u32", "i32", "f32", "u64"):
        for n, bits, kind in ((5000, 32, "ln"), (70000, 3, "ln"), (150000, 32, "eq"), (1, 32, "eq")):
            keys = inst.typed_keys(n, 40 + n + bits, t)
            if bits < 32:
                keys = (inst.uniform_keys(n, 41, bits=bits)).astype(keys.dtype)
            off = (inst.lognormal_offsets(n, 42, empty_frac=0.05) if kind == "ln"
                   else inst.equal_offsets_ragged(n, max(1, n // 7)))
            out.append((keys, off))
    return out


def _call_desc(pkg, torch, keys, off, vals):
    L = pkg.lib()
    n = len(keys)
    kt, gk = _guarded(torch, keys, 0x5A)
    dof = torch.from_numpy(off).cuda()
    st = torch.cuda.current_stream().cuda_stream
    kp = kt.data_ptr() + G * keys.itemsize
    if vals is None:
        rc = getattr(L, f"segsort_keys_{_SUF[keys.dtype]}_desc")(kp, n, dof.data_ptr(), len(off) - 1, st)
        vt = None
    else:
        vt, gv = _guarded(torch, vals, 0xA5)
        rc = getattr(L, f"segsort_pairs_{_SUF[keys.dtype]}_desc")(kp, vt.data_ptr() + G * 4, n,
                                                                 dof.data_ptr(), len(off) - 1, st)
    assert rc == pkg.SEGSORT_OK
    torch.cuda.synchronize()
    assert pkg.device_status() == pkg.SEGSORT_OK
    k = _unguard(kt, keys.dtype, n, gk)
    return (k, None) if vt is None else (k, _unguard(vt, np.uint32, n, gv))


def test_descending_pairs_match_oracle(pkg, cuda, inst, oracle):
    for keys, off in _instances(inst):
        vals = np.arange(len(keys), dtype=np.uint32)
        k, v = _call_desc(pkg, cuda, keys, off, vals)
        ek, ev = oracle.segsort_numpy(keys, off, vals, descending=True)
        assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)), (keys.dtype, len(keys))
        assert np.array_equal(v, ev), (keys.dtype, len(keys))


def test_descending_keys_only(pkg, cuda, inst, oracle):
    for keys, off in _instances(inst):
        if keys.dtype not in (np.uint32, np.float32):
            continue
        k, _ = _call_desc(pkg, cuda, keys, off, None)
        ek = oracle.segsort_numpy(keys, off, descending=True)
        assert np.array_equal(k.view(np.uint8), ek.view(np.uint8))


def test_descending_float_specials(pkg, cuda, oracle):
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40, -1e-40, 3.5, -3.5],
                        dtype=np.float32)
    keys = np.tile(specials, 500)
    off = np.array([0, 9, 4000, len(keys)], np.int32)
    vals = np.arange(len(keys), dtype=np.uint32)
    k, v = _call_desc(pkg, cuda, keys, off, vals)
    ek, ev = oracle.segsort_numpy(keys, off, vals, descending=True)
    assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)) and np.array_equal(v, ev)


@pytest.mark.parametrize("descending", [0, 1])
@pytest.mark.parametrize("kt", ["u32", "f32"])
def test_topk_matches_oracle(pkg, cuda, inst, oracle, descending, kt):
    torch = cuda
    L = pkg.lib()
    n = 200000
    keys = inst.typed_keys(n, 77, kt)
    off = inst.lognormal_offsets(n, 78, empty_frac=0.05)
    nseg = len(off) - 1
    vals = np.arange(n, dtype=np.uint32)
    for k in (1, 7, 300):
        dk = torch.from_numpy(keys.view(_VIEW[keys.dtype]).copy()).cuda()
        dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
        do = torch.from_numpy(off).cuda()
        fill_k = np.full(nseg * k, 0x7E7E7E7E, dtype=np.uint32).view(keys.dtype)
        ok = torch.from_numpy(fill_k.view(_VIEW[keys.dtype]).copy()).cuda()
        ov = torch.full((nseg * k,), -1, dtype=torch.int32, device="cuda")
        oc = torch.full((nseg,), -7, dtype=torch.int32, device="cuda")
        rc = getattr(L, f"segsort_pairs_{kt}_topk")(dk.data_ptr(), dv.data_ptr(), n, do.data_ptr(),
                                                  nseg, k, descending, ok.data_ptr(), ov.data_ptr(),
                                                  oc.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == pkg.SEGSORT_OK
        torch.cuda.synchronize()
        ek, ev = oracle.segsort_numpy(keys, off, vals, descending=bool(descending))
        got_k = ok.cpu().numpy().view(keys.dtype).reshape(nseg, k)
        got_v = ov.cpu().numpy().view(np.uint32).reshape(nseg, k)
        got_c = oc.cpu().numpy()
        lens = np.diff(off)
        assert np.array_equal(got_c, np.minimum(lens, k))
        for s in range(nseg):
            c = min(lens[s], k)
            b = off[s]
            assert np.array_equal(got_k[s, :c].view(np.uint8), ek[b:b + c].view(np.uint8)), (k, s)
            assert np.array_equal(got_v[s, :c], ev[b:b + c])
            assert np.array_equal(got_k[s, c:].view(np.uint32), np.full(k - c, 0x7E7E7E7E, np.uint32))
            assert np.all(got_v[s, c:] == 0xFFFFFFFF)
        # the input was sorted in place as well
        assert np.array_equal(dk.cpu().numpy().view(keys.dtype).view(np.uint8), ek.view(np.uint8))


def test_64bit_values_match_oracle(pkg, cuda, inst, oracle):
    torch = cuda
    L = pkg.lib()
    rng = np.random.default_rng(9)
    for keys, off in _instances(inst):
        n = len(keys)
        vals = rng.integers(0, 1 << 63, n, dtype=np.uint64) | np.uint64(1 << 63)
        kt, gk = _guarded(torch, keys, 0x33)
        vt, gv = _guarded(torch, vals, 0xC7)
        do = torch.from_numpy(off).cuda()
        rc = getattr(L, f"segsort_pairs_{_SUF[keys.dtype]}_v64")(
            kt.data_ptr() + G * keys.itemsize, vt.data_ptr() + G * 8, n, do.data_ptr(), len(off) - 1,
            torch.cuda.current_stream().cuda_stream)
        assert rc == pkg.SEGSORT_OK
        torch.cuda.synchronize()
        assert pkg.device_status() == pkg.SEGSORT_OK
        k = _unguard(kt, keys.dtype, n, gk)
        v = _unguard(vt, np.uint64, n, gv)
        ek, ev = oracle.segsort_numpy(keys, off, vals)
        assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)), (keys.dtype, n)
        assert np.array_equal(v, ev), (keys.dtype, n)


def _reduce_oracle(oracle, keys, off, vals):
    k, v = oracle.segsort_numpy(keys, off, vals)
    ok, osum, ocnt, ooff = [], [], [], []
    for s in range(len(off) - 1):
        ooff.append(len(ok))
        b, e = int(off[s]), int(off[s + 1])
        i = b
        while i < e:
            j = i
            while j < e and k[j] == k[i]:
                j += 1
            ok.append(k[i])
            osum.append(int(v[i:j].astype(np.uint64).sum()))
            ocnt.append(j - i)
            i = j
    ooff.append(len(ok))
    return (np.array(ok, np.uint32), np.array(osum, np.uint64), np.array(ocnt, np.uint32),
            np.array(ooff, np.int32), k)


def test_reduce_by_key_matches_oracle(pkg, cuda, inst, oracle):
    torch = cuda
    L = pkg.lib()
    rng = np.random.default_rng(3)
    cases = [
        (inst.uniform_keys(50000, 5, bits=6), inst.lognormal_offsets(50000, 6, empty_frac=0.05)),
        (inst.uniform_keys(20000, 7, bits=32), inst.equal_offsets_ragged(20000, 333)),
        (inst.uniform_keys(9000, 8, bits=1), np.array([5, 5, 100, 8000, 8000, 8990], np.int32)),
        (np.zeros(4096 * 3, np.uint32), np.array([0, 4096 * 3], np.int32)),
    ]
    for keys, off in cases:
        n = len(keys)
        vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
        dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
        do = torch.from_numpy(off).cuda()
        nseg = len(off) - 1
        ok = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        osum = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        ocnt = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        ooff = torch.full((nseg + 1,), -1, dtype=torch.int32, device="cuda")
        rc = L.segsort_pairs_u32_reduce_by_key(dk.data_ptr(), dv.data_ptr(), n, do.data_ptr(), nseg,
                                               ok.data_ptr(), osum.data_ptr(), ocnt.data_ptr(),
                                               ooff.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == pkg.SEGSORT_OK
        torch.cuda.synchronize()
        ek, es, ec, eo, sorted_keys = _reduce_oracle(oracle, keys, off, vals)
        runs = int(eo[-1])
        assert np.array_equal(ooff.cpu().numpy(), eo)
        assert np.array_equal(ok.cpu().numpy().view(np.uint32)[:runs], ek)
        assert np.array_equal(osum.cpu().numpy().view(np.uint64)[:runs], es)
        assert np.array_equal(ocnt.cpu().numpy().view(np.uint32)[:runs], ec)
        assert np.array_equal(dk.cpu().numpy().view(np.uint32), sorted_keys)
