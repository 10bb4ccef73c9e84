"""Failure detection on the GPU without a GPU fault: every device-side wait of
the sort kernels is bounded. Each self-test runs one wait's own device code on
a flag that nothing sets -- a look-back status word, a ring slot's completion
tag, a bulk copy's completion barrier, a bucket's running-prefix epoch, a
bucket tile's status, the 16-bit pass's work queue; the wait must run out,
the kernel must record LSB_ERR_DEVICE_TIMEOUT and return, and the context
must stay usable for the next sort."""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import to_dev, to_np

pytestmark = pytest.mark.gpu


def test_lookback_wait_runs_out_and_reports(lsb, cuda, oracle):
    t0 = time.perf_counter()
    status = lsb.selftest_wait_timeout()
    elapsed = time.perf_counter() - t0
    assert status == lsb.LSB_ERR_DEVICE_TIMEOUT
    assert elapsed < 60.0
    # the same process and context sort correctly afterwards
    a = oracle.generate(100003, oracle.DIST_UNIFORM, 77)
    A = to_dev(a, cuda)
    lsb.sort_pairs(A, cuda.empty_like(A), 16)
    assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a))


@pytest.mark.parametrize("which", ["ring_slot", "bulk_copy", "bucket_prefix", "bucket_lookback", "scheduler"])
def test_every_bounded_wait_runs_out_and_reports(lsb, cuda, oracle, which):
    t0 = time.perf_counter()
    status = lsb.selftest_wait(lsb.WAITS[which])
    elapsed = time.perf_counter() - t0
    assert status == lsb.LSB_ERR_DEVICE_TIMEOUT, which
    assert elapsed < 60.0
    a = oracle.generate(100003, oracle.DIST_ZIPF, 78)
    A = to_dev(a, cuda)
    lsb.sort_pairs(A, cuda.empty_like(A), 16)
    assert np.array_equal(to_np(A), oracle.stable_sort_by_key(a))
