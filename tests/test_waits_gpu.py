"""The failure path of the bounded device waits, without a GPU fault.

Every spin in the kernels (the grid barrier of the cooperative long-segment
kernel, the streamed tile kernel's mbarrier wait for its bulk copies, the
radix passes' look-back) gives up after a limit, records a timeout on the
device and returns, so a lost arrival can corrupt a result but never hang
the GPU.  segsort_selftest_wait_timeout launches, for each kind of wait, a
small kernel whose wait can never complete (a CTA that skips the barrier,
an mbarrier expecting bytes no copy supplies, a predecessor tile that never
publishes) with a limit of a few milliseconds.  The test checks that the
call returns, that segsort_device_status reports SEGSORT_ERR_TIMEOUT once,
and that the status reads clean after it was cleared.
"""
from __future__ import annotations

import time

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2], ids=["grid_barrier", "mbarrier", "look_back"])
def test_wait_that_never_completes_reports_timeout(pkg, cuda, which):
    L = pkg.lib()
    assert pkg.device_status(clear=True) in (pkg.SEGSORT_OK, pkg.SEGSORT_ERR_TIMEOUT)
    assert pkg.device_status(clear=True) == pkg.SEGSORT_OK
    t0 = time.perf_counter()
    assert L.segsort_selftest_wait_timeout(which) == pkg.SEGSORT_OK
    assert time.perf_counter() - t0 < 10.0
    assert pkg.device_status(clear=True) == pkg.SEGSORT_ERR_TIMEOUT
    assert pkg.device_status(clear=True) == pkg.SEGSORT_OK


def test_selftest_rejects_an_unknown_wait(pkg, cuda):
    assert pkg.lib().segsort_selftest_wait_timeout(7) == pkg.SEGSORT_ERR_INVALID_ARG


def test_sorting_after_a_timeout_is_exact(pkg, cuda, oracle, inst):
    """The context stays usable: a sort right after the self-test is exact."""
    import numpy as np
    from test_parity_gpu import check_both
    assert pkg.lib().segsort_selftest_wait_timeout(0) == pkg.SEGSORT_OK
    assert pkg.device_status(clear=True) == pkg.SEGSORT_ERR_TIMEOUT
    off = inst.diff_offsets(100000, 6, seed=81)
    check_both(pkg, cuda, oracle, inst.uniform_keys(100000, seed=81), off)
