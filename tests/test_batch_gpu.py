"""GPU parity of the batched form (segsort_pairs_batch and batch plans).

Bar: every instance of a batch comes out bit for bit as the oracle's stable
per-segment sort of that instance alone, and as the plain call on the same
instance; guard bands around every instance stay untouched.  The mix covers
every key type, CSR and heads-only offsets, instances that fit one tile,
instances with segments longer than the tile capacity and the long-segment
chunk, low-entropy keys, and empty instances.  The 64-instance mixed batch
of the benchmark (n up to 2^24 per instance) is checked against plain calls
element by element.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_VIEW = {np.dtype(np.uint32): np.int32, np.dtype(np.int32): np.int32,
         np.dtype(np.float32): np.float32, np.dtype(np.uint64): np.int64}
_CODE = {"u32": 0, "i32": 1, "f32": 2, "u64": 3}
GUARD = 5


class _DevInstance:
    """One instance in device memory, surrounded by guard bands."""

    def __init__(self, torch, keys, vals, off, key_type, heads=False):
        self.keys, self.vals, self.off, self.key_type, self.heads = keys, vals, off, key_type, heads
        self.n = len(keys)
        gk = np.full(GUARD, 0x3C, dtype=keys.dtype)
        gv = np.full(GUARD, 0xC3C3C3C3, dtype=np.uint32)
        self.gk, self.gv = gk, gv
        self.kbuf = torch.from_numpy(np.concatenate([gk, keys, gk]).view(_VIEW[keys.dtype])).cuda()
        self.vbuf = torch.from_numpy(np.concatenate([gv, vals, gv]).view(np.int32)).cuda()
        self.dof = torch.from_numpy(np.ascontiguousarray(off, dtype=np.int32)).cuda()
        self.kptr = self.kbuf.data_ptr() + GUARD * keys.itemsize
        self.vptr = self.vbuf.data_ptr() + GUARD * 4
        self.nseg = len(off) - (0 if heads else 1)

    def item(self, pkg):
        return pkg.BatchItem(_CODE[self.key_type], 1 if self.heads else 0, self.kptr, self.vptr,
                             self.n, self.dof.data_ptr(), self.nseg, 0)

    def reset(self, torch):
        self.kbuf.copy_(torch.from_numpy(np.concatenate([self.gk, self.keys, self.gk])
                                         .view(_VIEW[self.keys.dtype])))
        self.vbuf.copy_(torch.from_numpy(np.concatenate([self.gv, self.vals, self.gv]).view(np.int32)))

    def result(self):
        k = self.kbuf.cpu().numpy().view(self.keys.dtype)
        v = self.vbuf.cpu().numpy().view(np.uint32)
        assert np.array_equal(k[:GUARD].view(np.uint8), self.gk.view(np.uint8))
        assert np.array_equal(k[GUARD + self.n:].view(np.uint8), self.gk.view(np.uint8))
        assert np.array_equal(v[:GUARD], self.gv) and np.array_equal(v[GUARD + self.n:], self.gv)
        return k[GUARD:GUARD + self.n].copy(), v[GUARD:GUARD + self.n].copy()

    def plain(self, pkg, torch):
        """The same instance through its plain call, for comparison."""
        self.reset(torch)
        L = pkg.lib()
        st = torch.cuda.current_stream().cuda_stream
        if self.heads:
            rc = L.segsort_pairs_u32_heads(self.kptr, self.vptr, self.n, self.dof.data_ptr(),
                                           self.nseg, st)
        else:
            rc = getattr(L, f"segsort_pairs_{self.key_type}")(self.kptr, self.vptr, self.n,
                                                              self.dof.data_ptr(), self.nseg, st)
        assert rc == pkg.SEGSORT_OK
        torch.cuda.synchronize()
        return self.result()


def _mix(inst):
    """(keys, offsets, key_type, heads) of a mixed small batch."""
    cases = []
    sizes = [1, 100, 4096, 5000, 9000, 20000, 70000, 150000]
    types = ["u32", "i32", "f32", "u64"]
    seed = 900
    for i, n in enumerate(sizes):
        for t in types:
            seed += 1
            keys = inst.typed_keys(n, seed, t)
            if (i + len(t)) % 3 == 0:
                off = inst.lognormal_offsets(n, seed, empty_frac=0.05)
            elif n >= 8:
                off = inst.equal_offsets_ragged(n, max(1, n // (1 + seed % 5)))
            else:
                off = np.array([0, n], dtype=np.int32)
            cases.append((keys, off, t, False))
    # low-entropy keys in long segments (stability), heads-only offsets, empty instances
    cases.append((inst.uniform_keys(60000, 77, bits=3), np.array([0, 10, 50000, 60000], np.int32),
                  "u32", False))
    heads_off = inst.diff_offsets(30000, 9, seed=78)[:-1]
    cases.append((inst.uniform_keys(30000, 78, bits=5), heads_off, "u32", True))
    cases.append((np.zeros(0, np.uint32), np.array([0], np.int32), "u32", False))
    cases.append((inst.typed_keys(50, 79, "f32"), np.array([0], np.int32), "f32", False))
    return cases


def _oracle_of(oracle, keys, off, heads):
    csr = oracle.heads_to_csr(off, len(keys)) if heads else off
    return oracle.segsort_numpy(keys, csr, np.arange(len(keys), dtype=np.uint32))


@pytest.mark.parametrize("msd", [1, 0], ids=["msd_route", "lsd_route"])
def test_batch_mix_matches_oracle_and_plain(pkg, cuda, inst, oracle, msd):
    """With the MSD route on, the 64-bit key group (instances above 2^15
    keys) runs its two stages (per-instance expanded offsets)."""
    torch = cuda
    dev = [_DevInstance(torch, k, np.arange(len(k), dtype=np.uint32), o, t, h)
           for k, o, t, h in _mix(inst)]
    items = (pkg.BatchItem * len(dev))(*[d.item(pkg) for d in dev])
    with pkg.params({pkg.PARAM_MSD: msd}):
        rc = pkg.lib().segsort_pairs_batch(items, len(dev), torch.cuda.current_stream().cuda_stream)
    assert rc == pkg.SEGSORT_OK
    torch.cuda.synchronize()
    assert pkg.device_status() == pkg.SEGSORT_OK
    got = [d.result() for d in dev]
    for d, (k, v) in zip(dev, got):
        ek, ev = _oracle_of(oracle, d.keys, d.off, d.heads)
        assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)), (d.key_type, d.n)
        assert np.array_equal(v, ev), (d.key_type, d.n)
    for d, (k, v) in zip(dev, got):
        pk, pv = d.plain(pkg, torch)
        assert np.array_equal(k.view(np.uint8), pk.view(np.uint8)) and np.array_equal(v, pv)


def test_batch_plan_replays(pkg, cuda, inst, oracle):
    """A plan sorts what its buffers hold at each launch; two launches in a
    row on fresh inputs give the oracle's result both times."""
    torch = cuda
    cases = _mix(inst)[::3]
    dev = [_DevInstance(torch, k, np.arange(len(k), dtype=np.uint32), o, t, h) for k, o, t, h in cases]
    items = (pkg.BatchItem * len(dev))(*[d.item(pkg) for d in dev])
    L = pkg.lib()
    plan = ctypes.c_void_p()
    assert L.segsort_batch_plan_create(items, len(dev), ctypes.byref(plan)) == pkg.SEGSORT_OK
    try:
        assert L.segsort_batch_plan_workspace_bytes(plan) > 0
        st = torch.cuda.current_stream().cuda_stream
        for rep in range(2):
            for d in dev:
                d.reset(torch)
            assert L.segsort_batch_plan_launch(plan, st) == pkg.SEGSORT_OK
            torch.cuda.synchronize()
            assert pkg.device_status() == pkg.SEGSORT_OK
            for d in dev:
                k, v = d.result()
                ek, ev = _oracle_of(oracle, d.keys, d.off, d.heads)
                assert np.array_equal(k.view(np.uint8), ek.view(np.uint8)), (rep, d.key_type, d.n)
                assert np.array_equal(v, ev)
    finally:
        L.segsort_batch_plan_destroy(plan)


def test_batch_python_api(pkg, cuda, inst, oracle):
    torch = cuda
    specs = inst.batch_specs(count=6, seed=11, lo_log=12, hi_log=16,
                             key_types=("u32", "i32", "f32", "u64"))
    tensors, expect = [], []
    for s in specs:
        off, keys = inst.batch_instance(s)
        vals = np.arange(len(keys), dtype=np.uint32)
        tensors.append((torch.from_numpy(keys.view(_VIEW[keys.dtype])).cuda(),
                        torch.from_numpy(vals.view(np.int32)).cuda(),
                        torch.from_numpy(off).cuda(), s["key_type"]))
        expect.append(oracle.segsort_numpy(keys, off, vals))
    plan = pkg.BatchPlan(tensors)
    plan.launch()
    torch.cuda.synchronize()
    for (k, v, _, _), (ek, ev) in zip(tensors, expect):
        assert np.array_equal(k.cpu().numpy().view(np.uint8), ek.view(np.uint8))
        assert np.array_equal(v.cpu().numpy().view(np.uint32), ev)
    plan.close()


def test_batch_mixed_64_instances_match_plain_calls(pkg, cuda, inst):
    """The benchmark's 64-instance mixed batch (n log-uniform in
    [2^16, 2^24], u32/u64/f32 keys): batch output == plain calls, bit for bit."""
    torch = cuda
    specs = inst.batch_specs()
    dev = []
    for s in specs:
        off, keys = inst.batch_instance(s)
        dev.append(_DevInstance(torch, keys, np.arange(len(keys), dtype=np.uint32), off,
                                s["key_type"]))
    items = (pkg.BatchItem * len(dev))(*[d.item(pkg) for d in dev])
    L = pkg.lib()
    plan = ctypes.c_void_p()
    assert L.segsort_batch_plan_create(items, len(dev), ctypes.byref(plan)) == pkg.SEGSORT_OK
    try:
        assert L.segsort_batch_plan_launch(plan, torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        assert pkg.device_status() == pkg.SEGSORT_OK
        got = [d.result() for d in dev]
    finally:
        L.segsort_batch_plan_destroy(plan)
    for d, (k, v) in zip(dev, got):
        pk, pv = d.plain(pkg, torch)
        assert np.array_equal(k.view(np.uint8), pk.view(np.uint8)), (d.key_type, d.n)
        assert np.array_equal(v, pv), (d.key_type, d.n)
        del d.kbuf, d.vbuf


def test_batch_plan_tuner_caches_its_choice(pkg, cuda, inst, oracle, tmp_path):
    """The tuner measures the launch shapes, records the choice for the
    batch's class in the cache file, and a second plan of the same class
    takes it from the file; results stay exact."""
    torch = cuda
    cases = _mix(inst)[::2]
    dev = [_DevInstance(torch, k, np.arange(len(k), dtype=np.uint32), o, t, h) for k, o, t, h in cases]
    items = (pkg.BatchItem * len(dev))(*[d.item(pkg) for d in dev])
    L = pkg.lib()
    cache = tmp_path / "tune.txt"
    st = torch.cuda.current_stream().cuda_stream
    chosen = []
    for rep in range(2):
        plan = ctypes.c_void_p()
        assert L.segsort_batch_plan_create(items, len(dev), ctypes.byref(plan)) == pkg.SEGSORT_OK
        try:
            k = ctypes.c_int32()
            assert L.segsort_batch_plan_tune(plan, st, str(cache).encode(), ctypes.byref(k)) == 0
            assert 1 <= k.value <= 3
            chosen.append(k.value)
            for d in dev:
                d.reset(torch)
            assert L.segsort_batch_plan_launch(plan, st) == pkg.SEGSORT_OK
            torch.cuda.synchronize()
            assert pkg.device_status() == pkg.SEGSORT_OK
            for d in dev:
                kk, vv = d.result()
                ek, ev = _oracle_of(oracle, d.keys, d.off, d.heads)
                assert np.array_equal(kk.view(np.uint8), ek.view(np.uint8))
                assert np.array_equal(vv, ev)
        finally:
            L.segsort_batch_plan_destroy(plan)
    lines = cache.read_text().split("\n")
    assert len([ln for ln in lines if ln.strip()]) == 1  # measured once, then read back
    assert chosen[0] == chosen[1] == int(lines[0].split()[1])
