"""GPU: the served form (segsort_server_*) returns, for every request, bit for
bit the result of that request sorted alone, whatever else shares its batch.

Requests of mixed sizes (empty ones, single-tile ones, ones with segments
longer than the tile capacity) are submitted back to back so that the
server coalesces them; each result is compared with the oracle and with the
plain call on that request alone.  A budget that holds only a few requests
at a time forces admissions to wait for memory, and a request larger than
the whole budget is refused.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(inst, count, seed):
    out = []
    sizes = [0, 1, 37, 4096, 4097, 9000, 30000, 120000, 250000]
    for r in range(count):
        n = sizes[r % len(sizes)] if r < len(sizes) else int(
            2 ** (10 + 8 * inst._unit(inst.draw(seed, 8, r, 1))[0]))
        keys = inst.uniform_keys(n, seed + r, bits=32 if r % 4 else 6)
        if n == 0:
            off = np.array([0], np.int32)
        elif r % 3 == 0:
            off = inst.equal_offsets_ragged(n, max(1, n // 3))
        else:
            off = inst.lognormal_offsets(n, seed + r, empty_frac=0.03)
        out.append((keys, np.arange(n, dtype=np.uint32), off))
    return out


def _pinned(torch, a):
    t = torch.empty(len(a), dtype=torch.int32, pin_memory=True)
    t.numpy()[:] = a.view(np.int32)
    return t


def _plain_alone(pkg, torch, keys, vals, off):
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    do = torch.from_numpy(off).cuda()
    if len(keys):
        rc = pkg.lib().segsort_pairs_u32(dk.data_ptr(), dv.data_ptr(), len(keys), do.data_ptr(),
                                         len(off) - 1, torch.cuda.current_stream().cuda_stream)
        assert rc == pkg.SEGSORT_OK
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


def _serve(pkg, torch, reqs, budget, max_batch=0, depth=0):
    bufs = [(_pinned(torch, keys), _pinned(torch, vals), _pinned(torch, off),
             torch.zeros(len(keys), dtype=torch.int32, pin_memory=True),
             torch.zeros(len(keys), dtype=torch.int32, pin_memory=True))
            for keys, vals, off in reqs]
    srv = pkg.Server(budget, max_batch=max_batch, depth=depth)
    try:
        tickets = [srv.submit(*b) for b in bufs]  # back to back: they queue up
        lat = [srv.wait(t) for t in tickets]
        stats = srv.stats()
    finally:
        srv.close()
    assert all(x >= 0 for x in lat)
    return [(b[3].numpy().view(np.uint32).copy(), b[4].numpy().view(np.uint32).copy())
            for b in bufs], stats


def test_served_results_match_each_request_alone(pkg, cuda, inst, oracle):
    torch = cuda
    # A large first request keeps the one-batch pipeline busy while the
    # others arrive, so they are coalesced.
    big = 1 << 22
    reqs = [(inst.uniform_keys(big, 499), np.arange(big, dtype=np.uint32),
             inst.lognormal_offsets(big, 499))] + _requests(inst, 40, seed=500)
    got, stats = _serve(pkg, torch, reqs, budget=8 << 30, depth=1)
    assert stats["requests"] == len(reqs) and stats["status"] == pkg.SEGSORT_OK
    assert stats["batches"] < len(reqs)  # requests were coalesced
    assert pkg.device_status() == pkg.SEGSORT_OK
    for (keys, vals, off), (k, v) in zip(reqs, got):
        ek, ev = oracle.segsort_numpy(keys, off, vals)
        assert np.array_equal(k, ek) and np.array_equal(v, ev), len(keys)
        pk, pv = _plain_alone(pkg, torch, keys, vals, off)
        assert np.array_equal(k, pk) and np.array_equal(v, pv)


def test_served_under_a_small_budget_waits_for_memory(pkg, cuda, inst, oracle):
    """A budget that holds one of the largest requests but not two:
    admissions wait for memory to be released, and every result is still
    exact."""
    torch = cuda
    reqs = [r for r in _requests(inst, 24, seed=700) if len(r[0]) > 0]
    big = max(len(r[0]) for r in reqs)
    assert big >= 250000
    budget = int(1.2 * (20 * big + (1 << 20)))
    got, stats = _serve(pkg, torch, reqs, budget=budget, depth=2)
    assert stats["budget_waits"] > 0 and stats["peak_bytes"] <= budget
    for (keys, vals, off), (k, v) in zip(reqs, got):
        ek, ev = oracle.segsort_numpy(keys, off, vals)
        assert np.array_equal(k, ek) and np.array_equal(v, ev)
    srv = pkg.Server(1 << 20)
    try:
        keys, vals, off = max(reqs, key=lambda r: len(r[0]))
        out = np.zeros_like(keys)
        with pytest.raises(pkg.SegsortError) as e:
            srv.submit(keys, vals, off, out, out.copy())
        assert e.value.code == pkg.SEGSORT_ERR_TOO_LARGE
    finally:
        srv.close()


def test_served_one_request_per_batch(pkg, cuda, inst, oracle):
    torch = cuda
    reqs = _requests(inst, 10, seed=900)
    got, stats = _serve(pkg, torch, reqs, budget=8 << 30, max_batch=1, depth=1)
    assert stats["batches"] == len(reqs) and stats["max_batch"] == 1
    for (keys, vals, off), (k, v) in zip(reqs, got):
        ek, ev = oracle.segsort_numpy(keys, off, vals)
        assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_records_are_released_once_waited(pkg, cuda, inst):
    """Each ticket is waited for once; the server forgets a request after its
    wait returns, so a second wait on it is refused, while later tickets keep
    working after many earlier ones have been released."""
    import ctypes
    torch = cuda
    reqs = _requests(inst, 30, seed=301)
    bufs = [(_pinned(torch, keys), _pinned(torch, vals), _pinned(torch, off),
             torch.zeros(len(keys), dtype=torch.int32, pin_memory=True),
             torch.zeros(len(keys), dtype=torch.int32, pin_memory=True))
            for keys, vals, off in reqs]
    srv = pkg.Server(1 << 33)
    try:
        for rnd in range(3):  # three rounds of submit-all / wait-all
            tickets = [srv.submit(*[b.numpy() for b in bb]) for bb in bufs]
            for t in tickets:
                srv.wait(t)
            for t in tickets[:3]:
                rc = pkg.lib().segsort_server_wait(srv._h, t, None)
                assert rc == pkg.SEGSORT_ERR_INVALID_ARG
            for (keys, vals, off), bb in zip(reqs, bufs):
                ek, ev = _plain_alone(pkg, torch, keys, vals, off)
                assert np.array_equal(bb[3].numpy().view(np.uint32), ek)
                assert np.array_equal(bb[4].numpy().view(np.uint32), ev)
        st = srv.stats()
        assert st["requests"] == 90 and st["status"] == pkg.SEGSORT_OK
    finally:
        srv.close()
